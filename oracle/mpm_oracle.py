"""CPU oracle for diffmpm's explicit MPM step -- TEST INFRASTRUCTURE ONLY.

This module restates, in NumPy, the algorithm of geoelements/diffmpm's explicit
MPM time step (a JAX code that cannot run without JAX).  It is the checker for
the CUDA path: only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU
baseline leg may import it, and never as the thing measured or shipped.  The
product package ``diffmpm_gb300`` does not import it.

Every class and method cites the reference function it restates
(``diffmpm/<file>.py:<lines>``).  The class and method names follow the
reference so that the parity tests read like the reference's own tests.

Parity pinning.  The restatement is checked against every known answer of the
reference's unit tests (``tests/test_element.py``, ``tests/test_particle.py``,
``tests/test_material.py``) and against the three end-to-end benchmark goldens
(``benchmarks/2d/*/test_benchmark.py``) by ``tests/test_oracle_kat.py`` and
``tests/test_oracle_goldens.py``.

Arithmetic.  ``dtype`` selects float32 (the reference's JAX default) or float64
(the "error vs FP64" run).  Every operation is written so that NumPy rounds to
``dtype`` after each step, in the order the reference writes it.  Where the
reference's rounding depends on XLA internals that cannot be observed without
JAX, the restatement fixes one order and says so:

* P2G scatters accumulate in particle order (``np.add.at`` is sequential), which
  is what the reference's per-particle ``lax.fori_loop`` of ``.at[].add`` does.
* Small dot products (the 4-node sums of G2P and of the strain rate) are summed
  left to right over the element's nodes.
* The Jacobian ``dN/dxi^T . X`` of an axis-aligned element is taken at its exact
  value ``diag((x1 - x0)/2, (y1 - y0)/2)`` for the float node coordinates; its
  inverse is then ``diag(2/(x1 - x0), 2/(y1 - y0))`` rounded once.
* The element locate returns the element whose lower-left node is the largest
  node with ``x_n <= x_p`` and ``y_n <= y_p`` (``element.py:820-840``) but flags
  particles that are not strictly inside the mesh instead of reproducing the
  reference's wrap-around ids; ``MPMExplicit`` raises for them.

Two behaviours are build definitions, not restatements (the reference has no
counterpart): the ``Newtonian`` material, and a particle population that mixes
materials through per-particle material ids.
"""
from __future__ import annotations

import math
from collections import defaultdict
from typing import NamedTuple, Optional, Sequence

import numpy as np

__all__ = [
    "Nodes", "Linear1D", "Quadrilateral4Node", "Particles", "LinearElastic",
    "SimpleMaterial", "Newtonian", "Constraint", "NodalForce", "ParticleTraction",
    "ParticleVelocityConstraint", "Unit", "Linear", "Mesh1D", "Mesh2D", "USF", "USL", "MPMExplicit",
    "OutOfMeshError",
]

FLUSH = 1e-12  # the reference's flush threshold (element.py:186, particle.py:311)


class OutOfMeshError(ValueError):
    """A particle is not strictly inside the mesh (the step cannot place it)."""


def _c(x, dtype):
    return np.asarray(x, dtype=dtype)


def _flush(a):
    """``where(|a| < 1e-12, 0, a)`` (element.py:185-189, 198-202, 320-329)."""
    return np.where(np.abs(a) < FLUSH, np.zeros_like(a), a)


# ----------------------------------------------------------------------------
# Time functions (functions.py:7-49)
# ----------------------------------------------------------------------------
class Unit:
    """``Unit.value -> 1.0`` (functions.py:16-31)."""

    def __init__(self, id):
        self.id = id

    def value(self, x, dtype=np.float32):
        """functions.py:21-22"""
        return _c(1.0, dtype)


class Linear:
    """Piecewise-linear time function (functions.py:33-49, ``jnp.interp``).

    Linear interpolation between the bracketing table points
    ``f = f[i-1] + ((x - x[i-1]) / (x[i] - x[i-1])) * (f[i] - f[i-1])``,
    held constant outside the table, in ``dtype`` arithmetic.
    """

    def __init__(self, id, xvalues, fxvalues):
        self.id = id
        self.xvalues = np.asarray(xvalues, dtype=np.float64)
        self.fxvalues = np.asarray(fxvalues, dtype=np.float64)

    def value(self, x, dtype=np.float32):
        """``jnp.interp(x, xvalues, fxvalues)`` (functions.py:40-41)."""
        xp = self.xvalues.astype(dtype)
        fp = self.fxvalues.astype(dtype)
        x = _c(x, dtype)
        if x < xp[0]:
            return fp[0]
        if x > xp[-1]:
            return fp[-1]
        i = int(np.searchsorted(xp, x, side="right"))
        i = min(max(i, 1), len(xp) - 1)
        dx = xp[i] - xp[i - 1]
        if dx == 0:
            return fp[i - 1]
        return fp[i - 1] + ((x - xp[i - 1]) / dx) * (fp[i] - fp[i - 1])


# ----------------------------------------------------------------------------
# Boundary conditions and loads (constraint.py:4-44, forces.py:9-61)
# ----------------------------------------------------------------------------
class Constraint:
    """Velocity constraint (constraint.py:4-44)."""

    def __init__(self, dir: int, velocity: float):
        self.dir = dir
        self.velocity = velocity

    def apply(self, obj, ids):
        """Set velocity, momentum = m * v_bar and acceleration = 0 on ``ids``
        in direction ``dir`` (constraint.py:29-44)."""
        dt = obj.velocity.dtype
        ids = np.asarray(ids, dtype=np.int64).reshape(-1)
        v = _c(self.velocity, dt)
        obj.velocity[ids, :, self.dir] = v
        obj.momentum[ids, :, self.dir] = obj.mass[ids, :, 0] * v
        obj.acceleration[ids, :, self.dir] = 0


class NodalForce(NamedTuple):
    """Concentrated nodal force (forces.py:9-18)."""

    node_ids: object
    function: object
    dir: int
    force: float


class ParticleTraction(NamedTuple):
    """Particle surface traction (forces.py:26-41)."""

    pset: object
    pids: object
    function: object
    dir: int
    traction: float


class ParticleVelocityConstraint(NamedTuple):
    """Velocity ``velocity`` in direction ``dir`` of particles ``pids`` of the
    particle sets ``pset``, imposed after every particle velocity update (an
    extension: the reference leaves this as a TODO, scheme.py:67)."""

    pset: object
    pids: object
    dir: int
    velocity: float


# ----------------------------------------------------------------------------
# Materials (material.py:8-131) and the build's Newtonian definition
# ----------------------------------------------------------------------------
class _Material:
    """Material base (material.py:8-52)."""

    _props: tuple = ()
    incremental = True

    def validate_props(self, props):
        """KeyError naming a missing property (material.py:45-51)."""
        for key in self._props:
            if key not in props:
                raise KeyError(
                    f"'{key}' should be present in `material_properties` "
                    f"for {self.__class__.__name__} materials."
                )


class LinearElastic(_Material):
    """Linear elastic material (material.py:54-116).

    ``K = E/(3(1-2nu))``, ``G = E/(2(1+nu))``, ``a1 = K + 4G/3``,
    ``a2 = K - 2G/3`` in host float64, stored in ``dtype``; ``dsigma = D . deps``.
    """

    _props = ("density", "youngs_modulus", "poisson_ratio")

    def __init__(self, material_properties):
        self.validate_props(material_properties)
        E = float(material_properties["youngs_modulus"])
        nu = float(material_properties["poisson_ratio"])
        rho = float(material_properties["density"])
        K = E / (3 * (1 - 2 * nu))
        M = E * (1 - nu) / ((1 + nu) * (1 - 2 * nu))
        G = E / (2 * (1 + nu))
        self.properties = {
            **material_properties,
            "bulk_modulus": K,
            "pwave_velocity": math.sqrt(M / rho) if M / rho >= 0 else float("nan"),
            "swave_velocity": math.sqrt(G / rho) if G / rho >= 0 else float("nan"),
        }
        a1 = K + (4 * G / 3)
        a2 = K - (2 * G / 3)
        self._de64 = np.array(
            [
                [a1, a2, a2, 0, 0, 0],
                [a2, a1, a2, 0, 0, 0],
                [a2, a2, a1, 0, 0, 0],
                [0, 0, 0, G, 0, 0],
                [0, 0, 0, 0, G, 0],
                [0, 0, 0, 0, 0, G],
            ],
            dtype=np.float64,
        )
        self.coeffs = (a1, a2, G)

    def de(self, dtype):
        """The 6 x 6 elastic tensor of material.py:94-111 in ``dtype``."""
        return self._de64.astype(dtype)

    def compute_stress(self, dstrain):
        """``de @ dstrain`` with each row summed left to right
        (material.py:113-116)."""
        dtype = dstrain.dtype
        de = self.de(dtype)
        d = dstrain[..., 0]  # (N, 6)
        out = np.zeros_like(d)
        for r in range(6):
            acc = de[r, 0] * d[:, 0]
            for c in range(1, 6):
                acc = acc + de[r, c] * d[:, c]
            out[:, r] = acc
        return out[..., None]

    def __repr__(self):
        return f"LinearElastic(props={self.properties})"


class SimpleMaterial(_Material):
    """``dsigma = E * deps`` (material.py:119-131)."""

    _props = ("E", "density")

    def __init__(self, material_properties):
        self.validate_props(material_properties)
        self.properties = material_properties

    def compute_stress(self, dstrain):
        """material.py:130-131"""
        return dstrain * _c(self.properties["E"], dstrain.dtype)

    def __repr__(self):
        return f"SimpleMaterial(props={self.properties})"


class Newtonian(_Material):
    """Newtonian fluid -- a BUILD DEFINITION; the reference has no Newtonian.

    Total (not incremental) stress from the current strain rate and the
    volumetric strain at the element centroid ``eps_v``:

        p      = -K * eps_v                       (pressure, positive in compression)
        tr/3   = (rate_xx + rate_yy) / 3          (rate_zz = 0 in 2-D)
        s_xx   = -p + 2 mu (rate_xx - tr/3)
        s_yy   = -p + 2 mu (rate_yy - tr/3)
        s_zz   = -p - 2 mu tr/3
        s_xy   = mu * rate[3]                      (rate[3] is the engineering shear rate)
        s_yz   = s_xz = 0

    Float order: ``Kv = K*eps_v``; ``t3 = (rxx + ryy)/3``;
    ``s_xx = Kv + (2mu)*(rxx - t3)``; ``s_yy = Kv + (2mu)*(ryy - t3)``;
    ``s_zz = Kv - (2mu)*t3``; ``s_xy = mu*rate[3]``.
    """

    _props = ("density", "bulk_modulus", "dynamic_viscosity")
    incremental = False

    def __init__(self, material_properties):
        self.validate_props(material_properties)
        self.properties = dict(material_properties)

    def compute_total_stress(self, strain_rate, vsc):
        dt = strain_rate.dtype
        K = _c(self.properties["bulk_modulus"], dt)
        mu = _c(self.properties["dynamic_viscosity"], dt)
        twomu = _c(2.0 * float(self.properties["dynamic_viscosity"]), dt)
        r = strain_rate[:, :, 0]
        kv = K * vsc[:, 0]
        t3 = (r[:, 0] + r[:, 1]) / _c(3.0, dt)
        out = np.zeros_like(r)
        out[:, 0] = kv + twomu * (r[:, 0] - t3)
        out[:, 1] = kv + twomu * (r[:, 1] - t3)
        out[:, 2] = kv - twomu * t3
        out[:, 3] = mu * r[:, 3]
        return out[..., None]

    def __repr__(self):
        return f"Newtonian(props={self.properties})"


# ----------------------------------------------------------------------------
# Nodes (node.py:9-125)
# ----------------------------------------------------------------------------
class Nodes:
    """Nodal state (node.py:34-82): velocity, acceleration, momentum and forces
    start at zero, mass at one (node.py:64-71)."""

    def __init__(self, nnodes: int, loc, dtype=np.float32):
        loc = np.asarray(loc, dtype=dtype)
        if loc.ndim != 3:
            raise ValueError(f"`loc` should be of size (nnodes, 1, ndim); found {loc.shape}")
        self.nnodes = nnodes
        self.loc = loc
        self.velocity = np.zeros_like(loc)
        self.acceleration = np.zeros_like(loc)
        self.mass = np.ones((loc.shape[0], 1, 1), dtype=dtype)
        self.momentum = np.zeros_like(loc)
        self.f_int = np.zeros_like(loc)
        self.f_ext = np.zeros_like(loc)
        self.f_damp = np.zeros_like(loc)

    def __len__(self):
        return self.nnodes

    def get_total_force(self):
        """``f_int + f_ext + f_damp`` (node.py:123-125)."""
        return self.f_int + self.f_ext + self.f_damp


# ----------------------------------------------------------------------------
# Elements (element.py:21-909)
# ----------------------------------------------------------------------------
class _Element:
    """Shared P2G scatters and nodal update (element.py:121-340)."""

    nodes: Nodes
    dtype = np.float32

    # --- helpers -----------------------------------------------------------
    def _mapped(self, particles):
        N = self.shapefn(particles.reference_loc)[:, :, 0, 0]      # (Np, nn)
        ids = self.element_node_ids(particles.element_ids)           # (Np, nn)
        return N, ids

    def _scatter(self, target, ids, values):
        """Sequential ``target[ids] += values`` in particle-major order
        (the ``lax.fori_loop`` of ``.at[].add`` in element.py:138-152)."""
        np.add.at(target, ids.reshape(-1), values.reshape((-1,) + values.shape[2:]))

    # --- P2G (element.py:122-303) -------------------------------------------
    def compute_nodal_mass(self, particles):
        """m_i = sum_p N_i m_p, reset to 0 first (element.py:122-152)."""
        self.nodes.mass[:] = 0
        N, ids = self._mapped(particles)
        self._scatter(self.nodes.mass[:, 0, 0], ids, particles.mass[:, 0, 0][:, None] * N)

    def compute_nodal_momentum(self, particles):
        """p_i = sum_p N_i (m_p v_p), reset first, then flushed (element.py:154-189)."""
        self.nodes.momentum[:] = 0
        N, ids = self._mapped(particles)
        pmom = particles.mass * particles.velocity                  # (Np, 1, ndim)
        contrib = N[:, :, None] * pmom[:, 0, :][:, None, :]          # (Np, nn, ndim)
        self._scatter(self.nodes.momentum[:, 0, :], ids, contrib)
        self.nodes.momentum = _flush(self.nodes.momentum)

    def compute_velocity(self, particles):
        """v_i = p_i / m_i where m_i != 0, else keep v_i; flush (element.py:191-202)."""
        with np.errstate(divide="ignore", invalid="ignore"):
            v = np.where(self.nodes.mass == 0, self.nodes.velocity,
                         self.nodes.momentum / self.nodes.mass)
        self.nodes.velocity = _flush(v)

    def compute_external_force(self, particles):
        """f_ext = sum_p N_i f_ext,p, reset first (element.py:204-234)."""
        self.nodes.f_ext[:] = 0
        N, ids = self._mapped(particles)
        contrib = N[:, :, None] * particles.f_ext[:, 0, :][:, None, :]
        self._scatter(self.nodes.f_ext[:, 0, :], ids, contrib)

    def compute_body_force(self, particles, gravity):
        """f_ext += sum_p N_i (m_p g) (element.py:236-268)."""
        N, ids = self._mapped(particles)
        g = np.broadcast_to(_c(gravity, self.dtype).reshape(-1), (self.ndim,))
        mg = particles.mass[:, 0, 0][:, None] * g[None, :]           # (Np, ndim)
        contrib = N[:, :, None] * mg[:, None, :]
        self._scatter(self.nodes.f_ext[:, 0, :], ids, contrib)

    def apply_concentrated_nodal_forces(self, particles, curr_time):
        """f_ext[ids, dir] += f(t) * F (element.py:270-284)."""
        for cnf in self.concentrated_nodal_forces:
            factor = cnf.function.value(curr_time, self.dtype)
            ids = np.asarray(cnf.node_ids, dtype=np.int64).reshape(-1)
            np.add.at(self.nodes.f_ext[:, 0, cnf.dir], ids, factor * _c(cnf.force, self.dtype))

    def apply_particle_traction_forces(self, particles):
        """f_ext += sum_p N_i t_p (element.py:286-303)."""
        N, ids = self._mapped(particles)
        contrib = N[:, :, None] * particles.traction[:, 0, :][:, None, :]
        self._scatter(self.nodes.f_ext[:, 0, :], ids, contrib)

    def update_nodal_acceleration_velocity(self, particles, dt, *args):
        """a = nan_to_num(f/m); v += a dt; constraints; p = m v; flush v, a
        (element.py:305-329)."""
        total = self.nodes.get_total_force()
        with np.errstate(divide="ignore", invalid="ignore"):
            self.nodes.acceleration = np.nan_to_num(total / self.nodes.mass)
        self.nodes.velocity = self.nodes.velocity + self.nodes.acceleration * _c(dt, self.dtype)
        self.apply_boundary_constraints()
        self.nodes.momentum = self.nodes.mass * self.nodes.velocity
        self.nodes.velocity = _flush(self.nodes.velocity)
        self.nodes.acceleration = _flush(self.nodes.acceleration)

    def apply_boundary_constraints(self, *args):
        """Apply each (node_ids, Constraint) in list order (element.py:331-334)."""
        for ids, constraint in self.constraints:
            constraint.apply(self.nodes, ids)

    def id_to_node_loc(self, id):
        """element.py:47-62"""
        return self.nodes.loc[np.asarray(self.id_to_node_ids(id)).reshape(-1)]

    def id_to_node_vel(self, id):
        """element.py:64-79"""
        return self.nodes.velocity[np.asarray(self.id_to_node_ids(id)).reshape(-1)]


class Quadrilateral4Node(_Element):
    """2-D 4-node quadrilateral elements on a structured grid (element.py:603-909).

    Nodes are numbered row-major, ``id = j (nx + 1) + i`` at ``(i hx, j hy)``
    (element.py:663-690); element ``e`` has node ids
    ``[ll, ll + 1, ll + nx + 2, ll + nx + 1]``, ``ll = (e // nx)(nx + 1) + e % nx``
    (element.py:692-723).
    """

    ndim = 2
    nn = 4

    def __init__(self, nelements, total_elements, el_len, constraints, nodes=None,
                 concentrated_nodal_forces=(), initialized=None, volume=None,
                 dtype=np.float32):
        self.dtype = dtype
        self.nelements = tuple(int(n) for n in np.asarray(nelements).reshape(-1))
        self.nx, self.ny = self.nelements
        self.total_elements = int(total_elements)
        self.el_len = np.broadcast_to(np.asarray(el_len, dtype=dtype).reshape(-1), (2,)).copy()
        nx, ny = self.nx, self.ny
        self.node_x = np.arange(nx + 1).astype(dtype) * self.el_len[0]
        self.node_y = np.arange(ny + 1).astype(dtype) * self.el_len[1]
        if nodes is None:
            jj, ii = np.meshgrid(np.arange(ny + 1), np.arange(nx + 1), indexing="ij")
            loc = np.stack([self.node_x[ii.reshape(-1)], self.node_y[jj.reshape(-1)]], axis=-1)
            self.nodes = Nodes((nx + 1) * (ny + 1), loc.reshape(-1, 1, 2), dtype)
        else:
            self.nodes = nodes
        self.constraints = list(constraints)
        self.concentrated_nodal_forces = list(concentrated_nodal_forces)
        self.volume = (np.ones((self.total_elements, 1, 1), dtype=dtype)
                       if volume is None else np.asarray(volume, dtype=dtype))

    def id_to_node_ids(self, id):
        """element.py:692-723"""
        return self.element_node_ids(np.asarray(id)).reshape(4, 1)

    def element_node_ids(self, e):
        """Node ids of elements ``e``, counter-clockwise from the lower left
        (element.py:692-723, vectorised)."""
        e = np.asarray(e, dtype=np.int64)
        nx = self.nx
        ll = (e // nx) * (nx + 1) + e % nx
        return np.stack([ll, ll + 1, ll + nx + 2, ll + nx + 1], axis=-1)

    def shapefn(self, xi):
        """N = (1/4)(1 -/+ xi)(1 -/+ eta) in node order 0..3 (element.py:725-757)."""
        xi = np.asarray(xi)
        if xi.ndim != 3:
            raise ValueError(f"`xi` should be of size (npoints, 1, ndim); found {xi.shape}")
        x, y = xi[:, 0, 0], xi[:, 0, 1]
        q = _c(0.25, xi.dtype)
        res = np.stack([
            q * (1 - x) * (1 - y),
            q * (1 + x) * (1 - y),
            q * (1 + x) * (1 + y),
            q * (1 - x) * (1 + y),
        ], axis=1)
        return res[:, :, None, None]

    def _shapefn_natural_grad(self, xi):
        """dN/dxi (4 x 2) per point (element.py:759-789)."""
        xi = np.asarray(xi)
        pts = xi.reshape(-1, 2)
        x, y = pts[:, 0], pts[:, 1]
        q = _c(0.25, xi.dtype)
        g = np.stack([
            np.stack([-q * (1 - y), -q * (1 - x)], axis=-1),
            np.stack([q * (1 - y), -q * (1 + x)], axis=-1),
            np.stack([q * (1 + y), q * (1 + x)], axis=-1),
            np.stack([-q * (1 + y), q * (1 - x)], axis=-1),
        ], axis=1)
        return g  # (npoints, 4, 2)

    def shapefn_grad(self, xi, coords):
        """dN/dx = dN/dxi . inv(J)^T with J = dN/dxi^T . X (element.py:791-818).

        General form (any element geometry), used for the known-answer tests.
        """
        xi = np.asarray(xi)
        if xi.ndim != 3:
            raise ValueError(f"`x` should be of size (npoints, 1, ndim); found {xi.shape}")
        g = self._shapefn_natural_grad(xi)
        X = np.asarray(coords, dtype=g.dtype).reshape(-1, 4, 2)
        J = np.einsum("pna,pnb->pab", g, X)
        Jinv = np.linalg.inv(J).astype(g.dtype)
        return np.einsum("pna,pba->pnb", g, Jinv)

    def dn_dx(self, xi, element_ids):
        """``shapefn_grad`` on this axis-aligned mesh: ``dN/dx = dN/dxi * 2/(x1-x0)``,
        ``dN/dy = dN/deta * 2/(y1-y0)`` with the float node coordinates of the
        particle's element (J = diag((x1-x0)/2, (y1-y0)/2) exactly)."""
        i, j = self._ij(element_ids)
        rx = _c(2, self.dtype) / (self.node_x[i + 1] - self.node_x[i])
        ry = _c(2, self.dtype) / (self.node_y[j + 1] - self.node_y[j])
        g = self._shapefn_natural_grad(xi)
        return np.stack([g[:, :, 0] * rx[:, None], g[:, :, 1] * ry[:, None]], axis=-1)

    def _ij(self, e):
        e = np.asarray(e, dtype=np.int64)
        return e % self.nx, e // self.nx

    def locate(self, loc):
        """Element ids per element.py:820-840; -1 where the particle is not
        strictly inside the mesh (see the module docstring)."""
        x = loc[:, 0, 0]
        y = loc[:, 0, 1]
        i = np.searchsorted(self.node_x, x, side="right") - 1
        j = np.searchsorted(self.node_y, y, side="right") - 1
        ok = (i >= 0) & (i < self.nx) & (j >= 0) & (j < self.ny)
        return np.where(ok, j * self.nx + i, -1).astype(np.int32)

    def set_particle_element_ids(self, particles):
        """element.py:820-840"""
        particles.element_ids = self.locate(particles.loc)

    def compute_internal_force(self, particles):
        """f_int,i = -V_p [dNdx s_xx + dNdy s_xy, dNdy s_yy + dNdx s_xy]
        (element.py:842-901)."""
        self.nodes.f_int[:] = 0
        ids = self.element_node_ids(particles.element_ids)
        G = self.dn_dx(particles.reference_loc, particles.element_ids)   # (Np, 4, 2)
        s = particles.stress[:, :, 0]
        fx = G[:, :, 0] * s[:, 0:1] + G[:, :, 1] * s[:, 3:4]
        fy = G[:, :, 1] * s[:, 1:2] + G[:, :, 0] * s[:, 3:4]
        negv = -particles.volume[:, 0, 0][:, None]
        contrib = np.stack([negv * fx, negv * fy], axis=-1)              # (Np, 4, 2)
        self._scatter(self.nodes.f_int[:, 0, :], ids, contrib)

    def compute_volume(self, *args):
        """Bretschneider's formula with a = c = hy, b = d = hx (element.py:903-909)."""
        a = c = self.el_len[1]
        b = d = self.el_len[0]
        p = q = np.sqrt(a * a + b * b)
        four = _c(4, self.dtype)
        quarter = _c(0.25, self.dtype)
        t = a * a + c * c - b * b - d * d
        vol = quarter * np.sqrt(four * p * p * q * q - t * t)
        self.volume[:] = vol


class Linear1D(_Element):
    """1-D two-node line elements (element.py:343-600).

    Two behaviours are build definitions where the reference's 1-D path does not
    run as written: the element volume is ``x_{e+1} - x_e`` (the reference's
    ``ediff1d`` broadcast only works for one element, element.py:543-546), and
    the strain rate is ``[dN/dx . v, 0, 0, 0, 0, 0]`` (the reference indexes a
    1 x 1 matrix at ``[1, 1]``, particle.py:304-305).
    """

    ndim = 1
    nn = 2

    def __init__(self, nelements, total_elements, el_len, constraints, nodes=None,
                 concentrated_nodal_forces=(), initialized=None, volume=None,
                 dtype=np.float32):
        self.dtype = dtype
        self.nelements = int(np.asarray(nelements).reshape(-1)[0])
        self.nx = self.nelements
        self.total_elements = self.nelements
        self.el_len = _c(np.asarray(el_len).reshape(-1)[0], dtype)
        self.node_x = np.arange(self.nx + 1).astype(dtype) * self.el_len
        self.nodes = nodes if nodes is not None else Nodes(
            self.nx + 1, self.node_x.reshape(-1, 1, 1), dtype)
        self.constraints = list(constraints)
        self.concentrated_nodal_forces = list(concentrated_nodal_forces)
        self.volume = (np.ones((self.total_elements, 1, 1), dtype=dtype)
                       if volume is None else np.asarray(volume, dtype=dtype))

    def id_to_node_ids(self, id):
        """element.py:414-428"""
        return self.element_node_ids(np.asarray(id)).reshape(2, 1)

    def element_node_ids(self, e):
        """Node ids (e, e + 1) of elements ``e`` (element.py:414-428, vectorised)."""
        e = np.asarray(e, dtype=np.int64)
        return np.stack([e, e + 1], axis=-1)

    def shapefn(self, xi):
        """N = (1/2)(1 -/+ xi) (element.py:430-454)."""
        xi = np.asarray(xi)
        if xi.ndim != 3:
            raise ValueError(f"`xi` should be of size (npoints, 1, ndim); found {xi.shape}")
        h = _c(0.5, xi.dtype)
        x = xi[:, 0, 0]
        return np.stack([h * (1 - x), h * (1 + x)], axis=1)[:, :, None, None]

    def _shapefn_natural_grad(self, xi):
        """dN/dxi = [-1/2, 1/2] (element.py:456-486)."""
        xi = np.asarray(xi)
        n = xi.reshape(-1).shape[0]
        h = _c(0.5, xi.dtype)
        return np.tile(np.array([[-h], [h]], dtype=xi.dtype)[None], (n, 1, 1))

    def shapefn_grad(self, xi, coords):
        """element.py:488-515"""
        g = self._shapefn_natural_grad(xi)
        X = np.asarray(coords, dtype=g.dtype).reshape(-1, 2, 1)
        J = np.einsum("pna,pnb->pab", g, X)
        return g * (_c(1, g.dtype) / J)

    def dn_dx(self, xi, element_ids):
        """``shapefn_grad`` (element.py:488-515) with J = (x1 - x0)/2 exactly."""
        e = np.asarray(element_ids, dtype=np.int64)
        rx = _c(2, self.dtype) / (self.node_x[e + 1] - self.node_x[e])
        g = self._shapefn_natural_grad(xi)
        return g * rx[:, None, None]

    def locate(self, loc):
        """element.py:517-541: element i where x_i <= x < x_{i+1}, else -1."""
        x = loc[:, 0, 0]
        i = np.searchsorted(self.node_x, x, side="right") - 1
        ok = (i >= 0) & (i < self.nx)
        return np.where(ok, i, -1).astype(np.int32)

    def set_particle_element_ids(self, particles):
        """element.py:517-541"""
        particles.element_ids = self.locate(particles.loc)

    def compute_volume(self, *args):
        """Element length x_{e+1} - x_e in place of element.py:543-546 (see
        the class docstring)."""
        self.volume[:, 0, 0] = self.node_x[1:] - self.node_x[:-1]

    def compute_internal_force(self, particles):
        """f_int,i = (-V_p s_xx) dN_i/dx (element.py:548-600)."""
        self.nodes.f_int[:] = 0
        ids = self.element_node_ids(particles.element_ids)
        G = self.dn_dx(particles.reference_loc, particles.element_ids)[:, :, 0]  # (Np, 2)
        a = (-particles.volume[:, 0, 0]) * particles.stress[:, 0, 0]
        contrib = (a[:, None] * G)[:, :, None]
        self._scatter(self.nodes.f_int[:, 0, :], ids, contrib)


# ----------------------------------------------------------------------------
# Particles (particle.py:13-347)
# ----------------------------------------------------------------------------
class Particles:
    """Particle state (particle.py:16-91).

    ``material`` may be one material (the reference) or a list of materials
    with per-particle ``material_ids`` (a build extension: one population that
    mixes materials).  ``youngs_modulus`` optionally gives a per-particle E
    that replaces the material's (LinearElastic ``youngs_modulus``,
    SimpleMaterial ``E``; a build extension used by the differentiation
    workloads).
    """

    def __init__(self, loc, material, element_ids, initialized=None, data=None,
                 material_ids=None, youngs_modulus=None, dtype=np.float32):
        loc = np.array(loc, dtype=dtype)
        if loc.ndim != 3:
            raise ValueError(f"`loc` should be of size (nparticles, 1, ndim); found {loc.shape}")
        self.dtype = dtype
        self.loc = loc
        self.element_ids = np.asarray(element_ids, dtype=np.int32)
        self.materials = list(material) if isinstance(material, (list, tuple)) else [material]
        self.material = self.materials[0]
        n = loc.shape[0]
        self.material_ids = (np.zeros(n, dtype=np.int32) if material_ids is None
                             else np.asarray(material_ids, dtype=np.int32).reshape(n))
        self.youngs_modulus = None if youngs_modulus is None else np.asarray(
            youngs_modulus, dtype=np.float64).reshape(n)
        self.mass = np.ones((n, 1, 1), dtype=dtype)
        dens = np.array([float(m.properties["density"]) for m in self.materials])
        self.density = dens[self.material_ids].astype(dtype).reshape(n, 1, 1)
        self.volume = np.ones_like(self.mass)
        self.size = np.zeros_like(loc)
        self.velocity = np.zeros_like(loc)
        self.acceleration = np.zeros_like(loc)
        self.momentum = np.zeros_like(loc)
        self.strain = np.zeros((n, 6, 1), dtype=dtype)
        self.stress = np.zeros((n, 6, 1), dtype=dtype)
        self.strain_rate = np.zeros((n, 6, 1), dtype=dtype)
        self.dstrain = np.zeros((n, 6, 1), dtype=dtype)
        self.f_ext = np.zeros_like(loc)
        self.traction = np.zeros_like(loc)
        self.reference_loc = np.zeros_like(loc)
        self.dvolumetric_strain = np.zeros((n, 1), dtype=dtype)
        self.volumetric_strain_centroid = np.zeros((n, 1), dtype=dtype)

    def __len__(self):
        return self.loc.shape[0]

    def compute_volume(self, elements, total_elements):
        """V_p = V_el / count(e_p); size = V^(1/ndim); m_p = V_p rho_p
        (particle.py:158-178)."""
        e = self.element_ids
        cnt = np.bincount(e[e >= 0], minlength=elements.total_elements)
        ok = e >= 0
        vol = np.ones(len(self), dtype=self.dtype)
        vol[ok] = elements.volume[e[ok], 0, 0] / cnt[e[ok]].astype(self.dtype)
        self.volume[:, 0, 0] = vol
        ndim = self.loc.shape[-1]
        self.size[:] = (np.sqrt(self.volume) if ndim == 2 else self.volume)
        self.mass[:, 0, 0] = vol * self.density[:, 0, 0]

    def update_natural_coords(self, elements):
        """xi = (x - (x0 + x2)/2) * (2/(x2 - x0)) with the element's first and
        diagonally opposite nodes (particle.py:180-206)."""
        ids = elements.element_node_ids(self.element_ids)
        far = 2 if elements.ndim == 2 else 1
        t0 = elements.nodes.loc[ids[:, 0]]
        t2 = elements.nodes.loc[ids[:, far]]
        two = _c(2, self.dtype)
        self.reference_loc = (self.loc - (t0 + t2) / two) * (two / (t2 - t0))

    def update_position_velocity(self, elements, dt, velocity_update):
        """G2P (particle.py:208-247): v_hat = sum N v_i, a_hat = sum N a_i;
        v_p = v_hat if velocity_update else v_p + a_hat dt; x_p += v_hat dt."""
        N, ids = elements._mapped(self)
        nv = elements.nodes.velocity[ids][:, :, 0, :]       # (Np, nn, ndim)
        na = elements.nodes.acceleration[ids][:, :, 0, :]
        vh = N[:, 0, None] * nv[:, 0]
        ah = N[:, 0, None] * na[:, 0]
        for k in range(1, N.shape[1]):
            vh = vh + N[:, k, None] * nv[:, k]
            ah = ah + N[:, k, None] * na[:, k]
        dtc = _c(dt, self.dtype)
        if velocity_update:
            self.velocity[:, 0, :] = vh
        else:
            self.velocity[:, 0, :] = self.velocity[:, 0, :] + ah * dtc
        self.loc[:, 0, :] = self.loc[:, 0, :] + vh * dtc
        self.momentum = self.mass * self.velocity

    def _compute_strain_rate(self, dn_dx, elements):
        """[M00, M11, 0, M01 + M10, 0, 0] with M = dN/dx^T . v_el, flushed
        (particle.py:281-313)."""
        ids = elements.element_node_ids(self.element_ids)
        v = elements.nodes.velocity[ids][:, :, 0, :]          # (Np, nn, ndim)
        n = len(self)
        sr = np.zeros((n, 6, 1), dtype=self.dtype)
        if elements.ndim == 2:
            def msum(a, b):
                acc = dn_dx[:, 0, a] * v[:, 0, b]
                for k in range(1, dn_dx.shape[1]):
                    acc = acc + dn_dx[:, k, a] * v[:, k, b]
                return acc
            sr[:, 0, 0] = msum(0, 0)
            sr[:, 1, 0] = msum(1, 1)
            sr[:, 3, 0] = msum(0, 1) + msum(1, 0)
        else:
            acc = dn_dx[:, 0, 0] * v[:, 0, 0]
            acc = acc + dn_dx[:, 1, 0] * v[:, 1, 0]
            sr[:, 0, 0] = acc
        return _flush(sr)

    def compute_strain(self, elements, dt):
        """particle.py:249-279"""
        dtc = _c(dt, self.dtype)
        G = elements.dn_dx(self.reference_loc, self.element_ids)
        self.strain_rate = self._compute_strain_rate(G, elements)
        self.dstrain = self.strain_rate * dtc
        self.strain = self.strain + self.dstrain
        Gc = elements.dn_dx(np.zeros_like(self.loc), self.element_ids)
        src = self._compute_strain_rate(Gc, elements)
        ndim = self.loc.shape[-1]
        s = src[:, 0, :]
        for k in range(1, ndim):
            s = s + src[:, k, :]
        self.dvolumetric_strain = dtc * s
        self.volumetric_strain_centroid = self.volumetric_strain_centroid + self.dvolumetric_strain

    def compute_stress(self, *args):
        """sigma += material stress increment (particle.py:315-322); Newtonian
        particles take the material's total stress instead."""
        for m_id, mat in enumerate(self.materials):
            sel = self.material_ids == m_id
            if not sel.any():
                continue
            if isinstance(mat, Newtonian):
                self.stress[sel] = mat.compute_total_stress(
                    self.strain_rate[sel], self.volumetric_strain_centroid[sel])
            elif isinstance(mat, LinearElastic) and self.youngs_modulus is not None:
                self.stress[sel] = self.stress[sel] + _le_field_stress(
                    mat, self.youngs_modulus[sel], self.dstrain[sel])
            elif isinstance(mat, SimpleMaterial) and self.youngs_modulus is not None:
                # build extension: the per-particle E replaces the material's E
                E = self.youngs_modulus[sel].astype(self.dstrain.dtype)
                self.stress[sel] = self.stress[sel] + self.dstrain[sel] * E[:, None, None]
            else:
                self.stress[sel] = self.stress[sel] + mat.compute_stress(self.dstrain[sel])

    def update_volume(self, *args):
        """V *= 1 + dvol; rho /= 1 + dvol (particle.py:324-327)."""
        f = 1 + self.dvolumetric_strain
        self.volume[:, 0, :] = self.volume[:, 0, :] * f
        self.density[:, 0, :] = self.density[:, 0, :] / f

    def assign_traction(self, pids, dir, traction_):
        """t[pids, dir] += traction * V / size[dir] (particle.py:329-343)."""
        pids = np.asarray(pids, dtype=np.int64).reshape(-1)
        val = _c(traction_, self.dtype) * self.volume[pids, 0, 0] / self.size[pids, 0, dir]
        np.add.at(self.traction[:, 0, dir], pids, val)

    def zero_traction(self, *args):
        """particle.py:345-347"""
        self.traction[:] = 0


def _le_field_stress(mat, E, dstrain):
    """LinearElastic with a per-particle Young's modulus (build extension):
    ``a1 = E*c1``, ``a2 = E*c2``, ``G = E*c3`` with ``c1, c2, c3`` the float64
    coefficients of E for the material's Poisson ratio, each product rounded to
    ``dtype``; then the same row sums as ``LinearElastic.compute_stress``."""
    dtype = dstrain.dtype
    c1, c2, c3 = le_coefficients(float(mat.properties["poisson_ratio"]))
    Ed = E.astype(dtype)
    a1 = Ed * _c(c1, dtype)
    a2 = Ed * _c(c2, dtype)
    G = Ed * _c(c3, dtype)
    d = dstrain[:, :, 0]
    out = np.zeros_like(d)
    out[:, 0] = a1 * d[:, 0] + a2 * d[:, 1] + a2 * d[:, 2]
    out[:, 1] = a2 * d[:, 0] + a1 * d[:, 1] + a2 * d[:, 2]
    out[:, 2] = a2 * d[:, 0] + a2 * d[:, 1] + a1 * d[:, 2]
    out[:, 3] = G * d[:, 3]
    out[:, 4] = G * d[:, 4]
    out[:, 5] = G * d[:, 5]
    return out[..., None]


def le_coefficients(nu: float):
    """(a1, a2, G) per unit Young's modulus for Poisson ratio ``nu`` (float64),
    following material.py:95-111."""
    K = 1.0 / (3 * (1 - 2 * nu))
    G = 1.0 / (2 * (1 + nu))
    return K + 4 * G / 3, K - 2 * G / 3, G


# ----------------------------------------------------------------------------
# Mesh dispatch (mesh.py:13-126)
# ----------------------------------------------------------------------------
class _MeshBase:
    """mesh.py:13-94"""

    def __init__(self, config):
        self.particles = config["particles"]
        self.elements = config["elements"]
        self.particle_tractions = config.get("particle_surface_traction", [])
        self.particle_velocity_constraints = config.get("particle_velocity_constraints", [])

    def apply_particle_velocity_constraints(self):
        """v[pids, dir] = velocity for each entry in list order, after the
        particle velocity update (an extension: the reference leaves this
        step as a TODO, scheme.py:67); momentum follows the velocity."""
        dtype = self.elements.dtype
        for pc in self.particle_velocity_constraints:
            psets = pc.pset if isinstance(pc.pset, (list, tuple, np.ndarray)) else [pc.pset]
            for pset_id in psets:
                p = self.particles[int(pset_id)]
                ids = np.asarray(pc.pids, dtype=np.int64).reshape(-1)
                p.velocity[ids, 0, pc.dir] = _c(pc.velocity, dtype)
                p.momentum = p.mass * p.velocity

    def apply_on_elements(self, function, args=()):
        """mesh.py:31-43 -- the element method once per particle set."""
        f = getattr(self.elements, function)
        for pset in self.particles:
            f(pset, *args)

    def apply_on_particles(self, function, args=()):
        """mesh.py:45-58"""
        for pset in self.particles:
            getattr(pset, function)(self.elements, *args)

    def apply_traction_on_particles(self, curr_time):
        """mesh.py:60-77"""
        self.apply_on_particles("zero_traction")
        dtype = self.elements.dtype
        for pt in self.particle_tractions:
            val = pt.function.value(curr_time, dtype) * _c(pt.traction, dtype)
            psets = pt.pset if isinstance(pt.pset, (list, tuple, np.ndarray)) else [pt.pset]
            for pset_id in psets:
                self.particles[int(pset_id)].assign_traction(pt.pids, pt.dir, val)
        self.apply_on_elements("apply_particle_traction_forces")


class Mesh1D(_MeshBase):
    """mesh.py:96-109"""

    ndim = 1


class Mesh2D(_MeshBase):
    """mesh.py:113-126"""

    ndim = 2


# ----------------------------------------------------------------------------
# Schemes (scheme.py:13-133)
# ----------------------------------------------------------------------------
class _MPMScheme:
    """Phase order of scheme.py:16-75."""

    def __init__(self, mesh, dt, velocity_update):
        self.mesh = mesh
        self.dt = dt
        self.velocity_update = velocity_update

    def compute_nodal_kinematics(self):
        """scheme.py:22-29"""
        m = self.mesh
        m.apply_on_elements("set_particle_element_ids")
        m.apply_on_particles("update_natural_coords")
        m.apply_on_elements("compute_nodal_mass")
        m.apply_on_elements("compute_nodal_momentum")
        m.apply_on_elements("compute_velocity")
        m.apply_on_elements("apply_boundary_constraints")

    def compute_stress_strain(self):
        """scheme.py:31-35"""
        self.mesh.apply_on_particles("compute_strain", args=(self.dt,))
        self.mesh.apply_on_particles("update_volume")
        self.mesh.apply_on_particles("compute_stress")

    def compute_forces(self, gravity, step):
        """scheme.py:37-56 (t = step * dt in float arithmetic)."""
        dtype = self.mesh.elements.dtype
        t = _c(step, dtype) * _c(self.dt, dtype)
        m = self.mesh
        m.apply_on_elements("compute_external_force")
        m.apply_on_elements("compute_body_force", args=(gravity,))
        m.apply_traction_on_particles(t)
        m.apply_on_elements("apply_concentrated_nodal_forces", args=(t,))
        m.apply_on_elements("compute_internal_force")

    def compute_particle_kinematics(self):
        """scheme.py:58-67"""
        self.mesh.apply_on_elements("update_nodal_acceleration_velocity", args=(self.dt,))
        self.mesh.apply_on_particles("update_position_velocity",
                                     args=(self.dt, self.velocity_update))
        self.mesh.apply_particle_velocity_constraints()


class USF(_MPMScheme):
    """Stress update first (scheme.py:70-104)."""

    def precompute_stress_strain(self):
        """scheme.py:98-100"""
        self.compute_stress_strain()

    def postcompute_stress_strain(self):
        """scheme.py:102-104"""
        pass


class USL(_MPMScheme):
    """Stress update last (scheme.py:107-133)."""

    def precompute_stress_strain(self):
        """scheme.py:127-129"""
        pass

    def postcompute_stress_strain(self):
        """scheme.py:131-133"""
        self.compute_stress_strain()


# ----------------------------------------------------------------------------
# Solver (solver.py:19-222)
# ----------------------------------------------------------------------------
class MPMExplicit:
    """Explicit MPM driver (solver.py:19-222).

    ``solve_jit`` re-runs the constructor's volume set-up (R0: element ids,
    element volume, particle volume/size/mass) at the start of every step, as
    the reference's ``lax.fori_loop`` does by rebuilding the carry through
    ``tree_unflatten`` (solver.py:100-111, 213).  ``solve`` does not
    (solver.py:116-157).  Particles outside the mesh raise ``OutOfMeshError``.
    """

    _props = ("loc", "velocity", "stress", "strain")

    def __init__(self, mesh, dt, scheme="usf", velocity_update=False, sim_steps=1,
                 out_steps=1, out_dir="results/", writer_func=None):
        if scheme == "usf":
            self.mpm_scheme = USF(mesh, dt, velocity_update)
        elif scheme == "usl":
            self.mpm_scheme = USL(mesh, dt, velocity_update)
        else:
            raise ValueError(f"Please select scheme from ('usf', 'usl'). Found {scheme}")
        self.mesh = mesh
        self.dt = dt
        self.scheme = scheme
        self.velocity_update = velocity_update
        self.sim_steps = sim_steps
        self.out_steps = out_steps
        self.out_dir = out_dir
        self.writer_func = writer_func
        self._setup_volume()

    def _setup_volume(self):
        """solver.py:81-85"""
        m = self.mesh
        m.apply_on_elements("set_particle_element_ids")
        self._check_in_mesh()
        m.apply_on_elements("compute_volume")
        m.apply_on_particles("compute_volume", args=(m.elements.total_elements,))

    def _check_in_mesh(self):
        for pset in self.mesh.particles:
            if (pset.element_ids < 0).any():
                bad = int(np.argmax(pset.element_ids < 0))
                raise OutOfMeshError(f"particle {bad} is outside the mesh")

    def step(self, i, gravity, reinit=True):
        """One step: [R0], nodal kinematics, [USF stress], forces, particle
        kinematics, [USL stress] (solver.py:179-185)."""
        if reinit:
            self._setup_volume()
        s = self.mpm_scheme
        s.compute_nodal_kinematics()
        self._check_in_mesh()
        s.precompute_stress_strain()
        s.compute_forces(gravity, i)
        s.compute_particle_kinematics()
        s.postcompute_stress_strain()

    def _arrays(self):
        out = {}
        for name in self._props:
            out[name] = np.array([getattr(p, name).squeeze() for p in self.mesh.particles])
        return out

    def solve_jit(self, gravity):
        """solver.py:159-222; ``writer_func(arrays, step)`` is called after step
        ``i`` when ``i % out_steps == 0`` (solver.py:203-210)."""
        for i in range(self.sim_steps):
            self.step(i, gravity, reinit=True)
            if self.writer_func is not None and i % self.out_steps == 0:
                self.writer_func(self._arrays(), i)
        return {k: v.squeeze() for k, v in self._arrays().items()}

    def solve(self, gravity):
        """solver.py:116-157"""
        result = defaultdict(list)
        for i in range(self.sim_steps):
            self.step(i, gravity, reinit=False)
            for p in self.mesh.particles:
                result["position"].append(p.loc.copy())
                result["velocity"].append(p.velocity.copy())
                result["stress"].append(p.stress[:, :2, 0].copy())
                result["strain"].append(p.strain[:, :2, 0].copy())
        return {k: np.asarray(v) for k, v in result.items()}
