"""Material descriptors (the reference's diffmpm/material.py:8-131).

The stress updates run on the GPU; these classes validate and carry the
properties, and compute the derived constants the reference exposes.
"""
from __future__ import annotations

import math

from . import _lib


class Material:
    _props: tuple = ()
    kind = -1

    def __init__(self, material_properties):
        self.validate_props(material_properties)
        self.properties = dict(material_properties)

    def validate_props(self, material_properties):
        """Raise KeyError for a missing property (diffmpm/material.py:45-51)."""
        for key in self._props:
            if key not in material_properties:
                raise KeyError(f"'{key}' should be present in `material_properties` "
                               f"for {self.__class__.__name__} materials.")

    def to_c(self) -> "_lib.MpmMaterial":
        raise NotImplementedError

    def __repr__(self):
        return f"{self.__class__.__name__}(props={self.properties})"


class LinearElastic(Material):
    """Linear elastic material (diffmpm/material.py:54-116): D-matrix entries
    a1 = K + 4G/3, a2 = K - 2G/3 and G, computed in float64 and applied in float32."""

    _props = ("density", "youngs_modulus", "poisson_ratio")
    kind = _lib.LINEAR_ELASTIC

    def __init__(self, material_properties):
        super().__init__(material_properties)
        E = float(self.properties["youngs_modulus"])
        nu = float(self.properties["poisson_ratio"])
        rho = float(self.properties["density"])
        K = E / (3 * (1 - 2 * nu))
        M = E * (1 - nu) / ((1 + nu) * (1 - 2 * nu))
        G = E / (2 * (1 + nu))
        self.properties.update({
            "bulk_modulus": K,
            "pwave_velocity": math.sqrt(M / rho) if M / rho >= 0 else float("nan"),
            "swave_velocity": math.sqrt(G / rho) if G / rho >= 0 else float("nan"),
        })

    def to_c(self):
        p = self.properties
        return _lib.MpmMaterial(type=self.kind, density=float(p["density"]),
                                youngs_modulus=float(p["youngs_modulus"]),
                                poisson_ratio=float(p["poisson_ratio"]))


class SimpleMaterial(Material):
    """sigma += E * dstrain (diffmpm/material.py:119-131)."""

    _props = ("E", "density")
    kind = _lib.SIMPLE

    def to_c(self):
        p = self.properties
        return _lib.MpmMaterial(type=self.kind, density=float(p["density"]), E=float(p["E"]))


class Newtonian(Material):
    """Newtonian fluid.  The reference has no Newtonian material; this build
    defines it as a total (not incremental) stress

        s_ij = K eps_v delta_ij + 2 mu (rate_ij - tr(rate)/3 delta_ij)

    with eps_v the particle's volumetric strain at the element centroid
    (pressure p = -K eps_v) and rate the strain rate of the step; the shear
    components use the engineering shear rate (s_xy = mu * rate[3]) and
    s_yz = s_xz = 0."""

    _props = ("density", "bulk_modulus", "dynamic_viscosity")
    kind = _lib.NEWTONIAN

    def to_c(self):
        p = self.properties
        return _lib.MpmMaterial(type=self.kind, density=float(p["density"]),
                                bulk_modulus=float(p["bulk_modulus"]),
                                dynamic_viscosity=float(p["dynamic_viscosity"]))
