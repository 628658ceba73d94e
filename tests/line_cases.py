"""1-D (Linear1D) cases built with either API -- the oracle or the product."""
import numpy as np


def bar(api, nx=40, ppe=3, scheme="usf", velocity_update=False, sim_steps=50, dt=2e-4,
        material="linear", gravity=-9.81, seed=4, E=None, vshift=0.0, pvc=False, **kw):
    """A bar of ``nx`` elements on [0, 1], ``ppe`` particles per element over
    the middle 80 % of the elements with seeded jitter, node 0 fixed, a
    sinusoidal initial velocity (plus a uniform ``vshift``), gravity along the
    bar and a concentrated force ramp at the free end; ``pvc`` holds every
    4th particle's velocity with a particle velocity constraint."""
    h = 1.0 / nx
    rng = np.random.Generator(np.random.PCG64(seed))
    e0, e1 = int(0.1 * nx), int(0.9 * nx)
    off = (np.arange(ppe) + 0.5) / ppe
    x = ((np.arange(e0, e1)[:, None] + off[None, :]) * h).reshape(-1)
    x = x + rng.uniform(-0.1, 0.1, x.size) * h / ppe
    if material == "linear":
        mat = api.LinearElastic({"density": 1000.0, "youngs_modulus": 1e6, "poisson_ratio": 0.3})
    elif material == "newtonian":
        mat = api.Newtonian({"density": 1000.0, "bulk_modulus": 1e6, "dynamic_viscosity": 20.0})
    else:
        mat = api.SimpleMaterial({"density": 1000.0, "E": 1e6})
    fn = api.Linear(0, np.array([0.0, sim_steps * dt]), np.array([0.0, 1.0]))
    cnf = [api.NodalForce(node_ids=np.array([nx]), function=fn, dir=0, force=2.0)]
    cons = [(np.array([0]), api.Constraint(0, 0.0))]
    el = api.Linear1D(nx, nx, h, cons, concentrated_nodal_forces=cnf, **kw)
    ps = api.Particles(x.reshape(-1, 1, 1), mat, np.zeros(x.size, dtype=np.int32),
                       youngs_modulus=E, **kw)
    ps.velocity[:] = (vshift + 0.05 * np.sin(np.pi * x)).reshape(-1, 1, 1)
    mesh = api.Mesh1D({"particles": [ps], "elements": el, "particle_surface_traction": []})
    solver = api.MPMExplicit(mesh, dt, scheme=scheme, velocity_update=velocity_update,
                             sim_steps=sim_steps)
    if pvc:   # every 4th particle held at 0.02 m/s
        mesh.particle_velocity_constraints = [
            api.ParticleVelocityConstraint(pset=0, pids=np.arange(0, x.size, 4), dir=0, velocity=0.02)]
    return solver, np.array([gravity])


def point(api, E=100.0, scheme="usl", dt=0.01, sim_steps=1000, v0=0.1, **kw):
    """The reference's 1-D optimisation example (examples/optim_1d.py:14-26):
    one element of length 1 with node 0 fixed, one SimpleMaterial particle
    (density 1) at 0.5 moving at ``v0``, no gravity.  ``E`` is the material's
    modulus (a number) or a per-particle array."""
    Em = float(np.ravel(E)[0])
    mat = api.SimpleMaterial({"E": Em, "density": 1.0})
    cons = [(np.array([0]), api.Constraint(0, 0.0))]
    el = api.Linear1D(1, 1, 1.0, cons, **kw)
    Ep = None if np.ndim(E) == 0 else np.asarray(E, np.float64)
    ps = api.Particles(np.array([0.5]).reshape(1, 1, 1), mat, np.array([0]), youngs_modulus=Ep, **kw)
    ps.velocity[:] = v0
    mesh = api.Mesh1D({"particles": [ps], "elements": el, "particle_surface_traction": []})
    solver = api.MPMExplicit(mesh, dt, scheme=scheme, sim_steps=sim_steps)
    return solver, np.array([0.0])
