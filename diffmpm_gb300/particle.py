"""Particle state container (the reference's diffmpm/particle.py:13-136).

Host-side arrays in the reference's shapes and initial values
(particle.py:53-71).  A solve uploads them to the GPU.  Two build extensions:
``material`` may be a list of materials with per-particle ``material_ids`` (one
population mixing materials), and ``youngs_modulus`` gives particles their
own Young's modulus (replacing LinearElastic ``youngs_modulus`` or
SimpleMaterial ``E``).
"""
from __future__ import annotations

import numpy as np


class Particles:
    def __init__(self, loc, material, element_ids, initialized=None, data=None,
                 material_ids=None, youngs_modulus=None):
        loc = np.array(loc, dtype=np.float32)
        if loc.ndim != 3:
            raise ValueError(f"`loc` should be of size (nparticles, 1, ndim); found {loc.shape}")
        n = loc.shape[0]
        self.loc = loc
        self.element_ids = np.asarray(element_ids, dtype=np.int32)
        self.materials = list(material) if isinstance(material, (list, tuple)) else [material]
        self.material = self.materials[0]
        self.material_ids = (np.zeros(n, dtype=np.int32) if material_ids is None
                             else np.asarray(material_ids, dtype=np.int32).reshape(n))
        if self.material_ids.size and (self.material_ids.min() < 0
                                       or self.material_ids.max() >= len(self.materials)):
            raise ValueError("material_ids out of range")
        self.youngs_modulus = None if youngs_modulus is None else np.asarray(
            youngs_modulus, dtype=np.float32).reshape(n)
        dens = np.array([float(m.properties["density"]) for m in self.materials], dtype=np.float64)
        self.mass = np.ones((n, 1, 1), dtype=np.float32)
        self.density = dens.astype(np.float32)[self.material_ids].reshape(n, 1, 1)
        self.volume = np.ones_like(self.mass)
        self.size = np.zeros_like(loc)
        self.velocity = np.zeros_like(loc)
        self.acceleration = np.zeros_like(loc)
        self.momentum = np.zeros_like(loc)
        self.strain = np.zeros((n, 6, 1), dtype=np.float32)
        self.stress = np.zeros((n, 6, 1), dtype=np.float32)
        self.strain_rate = np.zeros((n, 6, 1), dtype=np.float32)
        self.dstrain = np.zeros((n, 6, 1), dtype=np.float32)
        self.f_ext = np.zeros_like(loc)
        self.traction = np.zeros_like(loc)
        self.reference_loc = np.zeros_like(loc)
        self.dvolumetric_strain = np.zeros((n, 1), dtype=np.float32)
        self.volumetric_strain_centroid = np.zeros((n, 1), dtype=np.float32)
        self.initialized = True

    def __len__(self):
        return self.loc.shape[0]

    def __repr__(self):
        return f"Particles(nparticles={len(self)})"
