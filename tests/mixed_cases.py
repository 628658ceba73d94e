"""A small mixed elastic + Newtonian population, built with either API -- the
oracle or the product -- for the adjoint tests on the CPU and the GPU."""
import numpy as np

from diffmpm_gb300 import workloads


def sheared(p):
    """Initial velocity (1.5 + 0.4 x + 0.8 y, 0.6 + 0.5 x - 0.3 y): particles
    change cell, and every strain rate is far from the flush threshold."""
    return np.stack([1.5 + 0.4 * p[:, 0] + 0.8 * p[:, 1], 0.6 + 0.5 * p[:, 0] - 0.3 * p[:, 1]],
                    axis=1)


def mixed_newtonian(api, scheme, dtype=np.float32, E=None):
    """16 x 16 mesh, Gauss-point particles over [0.1, 0.9] x [0, 0.6]: LinearElastic
    (per-particle E) left of x = 0.5, Newtonian right of it, sheared initial
    velocity, bottom fixed, gravity; USF at dt 1e-3 or USL at dt 2.5e-4, 24 steps."""
    n, h = 16, 1.0 / 16
    pts = workloads.gauss_points(2, 14, 0, 10, h)
    mid = (pts[:, 0] >= 0.5).astype(np.int32)
    mats = [api.LinearElastic({"density": 1000, "youngs_modulus": 1e6, "poisson_ratio": 0.3}),
            api.Newtonian({"density": 1000, "bulk_modulus": 5e5, "dynamic_viscosity": 50.0})]
    E0 = workloads.youngs_field(len(pts), 41) if E is None else E
    bottom = workloads._node_ids(n, n, lambda i, j: j == 0)
    cons = [(bottom, api.Constraint(0, 0.0)), (bottom, api.Constraint(1, 0.0))]
    dk = {} if dtype == np.float32 else {"dtype": dtype}   # (the oracle's float64 runs)
    el = api.Quadrilateral4Node((n, n), n * n, (h, h), cons, **dk)
    ps = api.Particles(pts.reshape(-1, 1, 2), mats, np.zeros(len(pts), dtype=np.int32),
                       material_ids=mid, youngs_modulus=E0, **dk)
    ps.velocity[:] = sheared(pts).reshape(-1, 1, 2)
    mesh = api.Mesh2D({"particles": [ps], "elements": el, "particle_surface_traction": []})
    dt = 1e-3 if scheme == "usf" else 2.5e-4
    solver = api.MPMExplicit(mesh, dt, scheme=scheme, sim_steps=24)
    return solver, np.array([0.0, -9.81]), E0


def simple_with_nodal_force(api, scheme, dtype=np.float32, E=None):
    """The same 16 x 16 block as ``mixed_newtonian`` in one SimpleMaterial
    (per-particle E) with a ramped concentrated force pulling down on three
    nodes of its top surface (nodes that carry mass), sheared initial velocity,
    bottom fixed, gravity; USF at dt 1e-3 or USL at dt 2.5e-4, 24 steps."""
    n, h = 16, 1.0 / 16
    pts = workloads.gauss_points(2, 14, 0, 10, h)
    mat = api.SimpleMaterial({"density": 1000, "E": 1e6})
    E0 = workloads.youngs_field(len(pts), 43) if E is None else E
    bottom = workloads._node_ids(n, n, lambda i, j: j == 0)
    cons = [(bottom, api.Constraint(0, 0.0)), (bottom, api.Constraint(1, 0.0))]
    dt = 1e-3 if scheme == "usf" else 2.5e-4
    ramp = api.Linear(0, np.array([0.0, 24 * dt]), np.array([0.0, 1.0]))
    top = np.array([10 * (n + 1) + i for i in (6, 8, 10)])
    cnf = [api.NodalForce(node_ids=top, function=ramp, dir=1, force=-50.0)]
    dk = {} if dtype == np.float32 else {"dtype": dtype}
    el = api.Quadrilateral4Node((n, n), n * n, (h, h), cons, concentrated_nodal_forces=cnf, **dk)
    ps = api.Particles(pts.reshape(-1, 1, 2), mat, np.zeros(len(pts), dtype=np.int32),
                       youngs_modulus=E0, **dk)
    ps.velocity[:] = sheared(pts).reshape(-1, 1, 2)
    mesh = api.Mesh2D({"particles": [ps], "elements": el, "particle_surface_traction": []})
    solver = api.MPMExplicit(mesh, dt, scheme=scheme, sim_steps=24)
    return solver, np.array([0.0, -9.81]), E0
