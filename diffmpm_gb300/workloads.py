"""Synthetic workloads of the benchmark configurations.

Each builder returns ``(solver, gravity, info)`` for an API module ``api`` that
exposes the reference's class names (this package, or any restatement with the
same surface), so that the same input can be built for two implementations.
Inputs are seeded (NumPy PCG64); no dataset is involved.

* ``plain_small``  10 x 10 Q4 mesh on [0,1]^2, 2 x 2 Gauss-point particles in
  the cells covering [0.2, 0.8]^2 (144 particles), LinearElastic E=1e4,
  nu=0.3, rho=1000, gravity (0, -9.81), nodes at y=0 fixed in x and y,
  dt=1e-4, USF, 1000 steps.
* ``plain_scaleup``  n x n mesh (n=1024 at full size) on [0,1]^2, 4 Gauss-point
  particles per cell filling x in [0, 0.5], y in [0, 1], jittered uniformly by
  +-0.1 h per component, LinearElastic E=1e6, nu=0.25, rho=2000, gravity,
  roller walls (x fixed at x=0 and x=1), bottom fixed, dt=1e-6, 500 steps,
  USF or USL.
* ``differentiation``  n x n mesh (n=256 at full size), 4 Gauss-point particles
  per cell in the cells whose centres lie in [0.1, 0.9] x [0, 0.6] (125,664
  particles at n=256), per-particle Young's modulus 1e6 exp(0.5 z), z ~ N(0,1)
  seeded, nu=0.3, rho=1000, gravity, bottom fixed, USF, dt=5e-6, 2000 steps.
* ``batch_specs`` / ``batch_member``  independent simulations of uneven size
  (512 at full size): mesh side uniform in {32, ..., 256} over [0, 0.05 m]^2,
  4 Gauss-point particles per cell in a seeded random rectangle of cells
  covering 20-60% of the domain, resting on the fixed bottom and kept 5% of
  the width from the side walls and the top, E log-uniform in [1e5, 1e8],
  nu uniform in [0.2, 0.35], rho=1500, gravity, dt = 0.3 h / v_p with the
  P-wave velocity of diffmpm/material.py:73-81, USF, velocity_update=False.
  The domain size is not part of the configuration; on [0, 1 m]^2 the softest
  blocks sag by more than a cell under gravity, their free surfaces leave
  nodes with vanishing mass, and the reference's step (a = nan_to_num(f/m),
  diffmpm/element.py:311) blows up within 1000 steps (in the float32 oracle:
  member 86 leaves the mesh at step 963; member 9 reaches 2991 m/s at step
  799).  At 0.05 m the sag stays below a tenth of a cell and all 512 members
  run 1000 steps.  Step cost does not depend on the domain size.
* ``mixed_large``  n x n mesh (n=4096 at full size), an elastic block
  x in [0.125, 0.375] and a Newtonian block x in [0.625, 0.875], both
  y in [0, 0.5], 4 Gauss points per cell, elastic E=5e6, nu=0.3, rho=1800,
  fluid K=2e6, mu=1e-3, rho=1000, initial velocities N(0, 0.01^2), gravity,
  roller walls and fixed bottom, USL, dt=2e-7, 200 steps.
"""
from __future__ import annotations

import numpy as np

GAUSS = 1.0 / (2.0 * np.sqrt(3.0))   # Gauss offset from the cell centre, in cells


def gauss_points(i0, i1, j0, j1, h):
    """Particles at the 2 x 2 Gauss points of cells [i0,i1) x [j0,j1) (float64),
    ordered cell by cell (row-major), 4 per cell."""
    ii, jj = np.meshgrid(np.arange(i0, i1), np.arange(j0, j1), indexing="xy")
    cx = (ii.reshape(-1) + 0.5) * h
    cy = (jj.reshape(-1) + 0.5) * h
    off = np.array([[-GAUSS, -GAUSS], [GAUSS, -GAUSS], [-GAUSS, GAUSS], [GAUSS, GAUSS]]) * h
    pts = np.stack([cx, cy], axis=-1)[:, None, :] + off[None, :, :]
    return pts.reshape(-1, 2)


def _node_ids(n_x, n_y, pred):
    ii, jj = np.meshgrid(np.arange(n_x + 1), np.arange(n_y + 1), indexing="xy")
    ii, jj = ii.reshape(-1), jj.reshape(-1)
    return np.nonzero(pred(ii, jj))[0].astype(np.int64)


def _mesh(api, n, h, constraints, kw):
    return api.Quadrilateral4Node((n, n), n * n, (h, h), constraints, **kw)


def plain_small(api, sim_steps=1000, dt=1e-4, velocity=None, velocity_update=False, **kw):
    n, h = 10, 0.1
    pts = gauss_points(2, 8, 2, 8, h)
    mat = api.LinearElastic({"density": 1000, "youngs_modulus": 1e4, "poisson_ratio": 0.3})
    bottom = _node_ids(n, n, lambda i, j: j == 0)
    cons = [(bottom, api.Constraint(0, 0.0)), (bottom, api.Constraint(1, 0.0))]
    el = _mesh(api, n, h, cons, kw)
    ps = api.Particles(pts.reshape(-1, 1, 2), mat, np.zeros(len(pts), dtype=np.int32), **kw)
    if velocity is not None:
        ps.velocity[:] = np.asarray(velocity, dtype=np.float64).reshape(1, 1, 2)
    mesh = api.Mesh2D({"particles": [ps], "elements": el, "particle_surface_traction": []})
    solver = api.MPMExplicit(mesh, dt, scheme="usf", velocity_update=velocity_update,
                             sim_steps=sim_steps)
    return solver, np.array([0.0, -9.81]), {"workload": "plain_small", "n": n, "np": len(pts)}


def _rollers_and_bottom(api, n):
    walls = _node_ids(n, n, lambda i, j: (i == 0) | (i == n))
    bottom = _node_ids(n, n, lambda i, j: j == 0)
    return [(walls, api.Constraint(0, 0.0)), (bottom, api.Constraint(0, 0.0)),
            (bottom, api.Constraint(1, 0.0))]


def plain_scaleup(api, n=1024, scheme="usf", sim_steps=500, seed=2024, rows=None, **kw):
    """``rows`` keeps only the particles of the first ``rows`` cell rows (a
    bounded sample of the same workload on the same mesh)."""
    h = 1.0 / n
    pts = gauss_points(0, n // 2, 0, n if rows is None else rows, h)
    rng = np.random.Generator(np.random.PCG64(seed))
    pts = pts + rng.uniform(-0.1 * h, 0.1 * h, size=pts.shape)
    mat = api.LinearElastic({"density": 2000, "youngs_modulus": 1e6, "poisson_ratio": 0.25})
    el = _mesh(api, n, h, _rollers_and_bottom(api, n), kw)
    ps = api.Particles(pts.reshape(-1, 1, 2), mat, np.zeros(len(pts), dtype=np.int32), **kw)
    mesh = api.Mesh2D({"particles": [ps], "elements": el, "particle_surface_traction": []})
    solver = api.MPMExplicit(mesh, 1e-6, scheme=scheme, velocity_update=False, sim_steps=sim_steps)
    return solver, np.array([0.0, -9.81]), {"workload": f"plain_scaleup_{scheme}", "n": n,
                                             "np": len(pts), "seed": seed}


def youngs_field(npart, seed, median=1e6, sigma_log=0.5):
    """Log-normal per-particle Young's modulus, median * exp(sigma_log z)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    return median * np.exp(sigma_log * rng.normal(size=npart))


def differentiation(api, n=256, sim_steps=2000, dt=5e-6, seed=101, velocity=None, E=None,
                    scheme="usf", traction=None, **kw):
    """``E`` overrides the seeded field; ``velocity`` sets the initial particle
    velocity (used by small test variants to make particles change cell): a
    2-vector for all particles, or a function of the (n, 2) positions;
    ``scheme`` (USF in the configuration) lets tests differentiate USL;
    ``traction`` = (dir, value) puts a particle traction on the top layer of
    particles, ramped linearly from 0 to ``value`` over the run (tests)."""
    h = 1.0 / n
    i0 = int(np.ceil(0.1 * n - 0.5))
    i1 = int(np.floor(0.9 * n - 0.5)) + 1
    j1 = int(np.floor(0.6 * n - 0.5)) + 1
    pts = gauss_points(i0, i1, 0, j1, h)
    E = youngs_field(len(pts), seed) if E is None else np.asarray(E, dtype=np.float64)
    mat = api.LinearElastic({"density": 1000, "youngs_modulus": 1e6, "poisson_ratio": 0.3})
    bottom = _node_ids(n, n, lambda i, j: j == 0)
    cons = [(bottom, api.Constraint(0, 0.0)), (bottom, api.Constraint(1, 0.0))]
    el = _mesh(api, n, h, cons, kw)
    ps = api.Particles(pts.reshape(-1, 1, 2), mat, np.zeros(len(pts), dtype=np.int32),
                       youngs_modulus=E, **kw)
    if velocity is not None:
        v = velocity(pts) if callable(velocity) else velocity
        ps.velocity[:] = np.broadcast_to(np.asarray(v, dtype=np.float64), pts.shape).reshape(-1, 1, 2)
    tractions = []
    if traction is not None:
        top = np.nonzero(pts[:, 1] > pts[:, 1].max() - 0.5 * h)[0]
        ramp = api.Linear(0, np.array([0.0, sim_steps * dt]), np.array([0.0, 1.0]))
        tractions = [api.ParticleTraction(0, top, ramp, int(traction[0]), float(traction[1]))]
    mesh = api.Mesh2D({"particles": [ps], "elements": el, "particle_surface_traction": tractions})
    solver = api.MPMExplicit(mesh, dt, scheme=scheme, velocity_update=False, sim_steps=sim_steps)
    return solver, np.array([0.0, -9.81]), {"workload": "differentiation", "n": n, "np": len(pts),
                                             "seed": seed, "E": E}


def batch_specs(nsims=512, seed=5, sides=(32, 256), area=(0.2, 0.6), E=(1e5, 1e8),
                nu=(0.2, 0.35), rho=1500.0, cfl=0.3, domain=0.05, velocity_update=False):
    """Seeded parameters of the batch members (plain dicts); the mesh covers
    [0, domain]^2."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for _ in range(nsims):
        n = int(rng.integers(sides[0], sides[1] + 1))
        a = rng.uniform(*area)
        aspect = np.exp(rng.uniform(np.log(0.5), np.log(2.0)))
        margin = int(np.ceil(0.05 * n))
        w = min(0.9, np.sqrt(a * aspect))
        hgt = min(0.9, a / w)
        wc = max(1, min(n - 2 * margin, int(round(w * n))))
        hc = max(1, min(n - margin, int(round(hgt * n))))
        i0 = int(rng.integers(margin, n - margin - wc + 1))
        Ek = float(np.exp(rng.uniform(np.log(E[0]), np.log(E[1]))))
        nuk = float(rng.uniform(*nu))
        M = Ek * (1 - nuk) / ((1 + nuk) * (1 - 2 * nuk))
        dt = cfl * (domain / n) / np.sqrt(M / rho)
        out.append({"side": n, "cells": (i0, i0 + wc, 0, hc), "E": Ek, "nu": nuk, "rho": rho,
                    "dt": float(dt), "np": 4 * wc * hc, "domain": domain,
                    "velocity_update": bool(velocity_update)})
    return out


def batch_member(api, spec, sim_steps=1000, **kw):
    n = spec["side"]
    h = spec["domain"] / n
    pts = gauss_points(*spec["cells"], h)
    mat = api.LinearElastic({"density": spec["rho"], "youngs_modulus": spec["E"],
                             "poisson_ratio": spec["nu"]})
    bottom = _node_ids(n, n, lambda i, j: j == 0)
    cons = [(bottom, api.Constraint(0, 0.0)), (bottom, api.Constraint(1, 0.0))]
    el = _mesh(api, n, h, cons, kw)
    ps = api.Particles(pts.reshape(-1, 1, 2), mat, np.zeros(len(pts), dtype=np.int32), **kw)
    mesh = api.Mesh2D({"particles": [ps], "elements": el, "particle_surface_traction": []})
    solver = api.MPMExplicit(mesh, spec["dt"], scheme="usf",
                             velocity_update=spec["velocity_update"], sim_steps=sim_steps)
    return solver, np.array([0.0, -9.81]), {"workload": "batch_member", "n": n, "np": len(pts)}


def mixed_large(api, n=4096, sim_steps=200, seed=7, **kw):
    h = 1.0 / n
    a0, a1 = int(round(0.125 * n)), int(round(0.375 * n))
    b0, b1 = int(round(0.625 * n)), int(round(0.875 * n))
    top = int(round(0.5 * n))
    elastic = gauss_points(a0, a1, 0, top, h)
    fluid = gauss_points(b0, b1, 0, top, h)
    pts = np.concatenate([elastic, fluid])
    mid = np.concatenate([np.zeros(len(elastic), np.int32), np.ones(len(fluid), np.int32)])
    mats = [api.LinearElastic({"density": 1800, "youngs_modulus": 5e6, "poisson_ratio": 0.3}),
            api.Newtonian({"density": 1000, "bulk_modulus": 2e6, "dynamic_viscosity": 1e-3})]
    rng = np.random.Generator(np.random.PCG64(seed))
    vel = rng.normal(0.0, 0.01, size=pts.shape)
    el = _mesh(api, n, h, _rollers_and_bottom(api, n), kw)
    ps = api.Particles(pts.reshape(-1, 1, 2), mats, np.zeros(len(pts), dtype=np.int32),
                       material_ids=mid, **kw)
    ps.velocity[:] = vel.reshape(-1, 1, 2)
    mesh = api.Mesh2D({"particles": [ps], "elements": el, "particle_surface_traction": []})
    solver = api.MPMExplicit(mesh, 2e-7, scheme="usl", velocity_update=False, sim_steps=sim_steps)
    return solver, np.array([0.0, -9.81]), {"workload": "mixed_large", "n": n, "np": len(pts),
                                             "seed": seed}


def particle_steps_bytes(np_, nn):
    """Algorithmic bytes of one step: 104 B of particle state read and written
    once per particle plus 72 B per node (the minimal unique float32 traffic)."""
    return 104.0 * np_ + 72.0 * nn
