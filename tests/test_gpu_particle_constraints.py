"""Particle velocity constraints (an extension; the reference leaves them as a
TODO at diffmpm/scheme.py:67): the GPU against the oracle's definition."""
import numpy as np
import pytest

import diffmpm_gb300 as D
from diffmpm_gb300 import workloads
from oracle import mpm_oracle as O
import line_cases as L

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)


def close_stress(a, b, tol=1e-4, floor=1e-3):
    """Relative tolerance, or the round-off floor of 1 mPa per particle for a
    stress that is exactly zero in exact arithmetic (the first USL step of a
    block at rest: uniform nodal velocities)."""
    d = np.linalg.norm(np.asarray(a, np.float64) - np.asarray(b, np.float64))
    return rel(a, b) <= tol or d <= floor * np.sqrt(np.size(a))


def constrained(api, solver, n):
    """Every 7th particle: dir 0 -> 0.02; every 5th: dir 1 -> -0.01 (the
    particles in both lists take both)."""
    pcs = [api.ParticleVelocityConstraint(pset=0, pids=np.arange(0, n, 7), dir=0, velocity=0.02),
           api.ParticleVelocityConstraint(pset=0, pids=np.arange(0, n, 5), dir=1, velocity=-0.01)]
    solver.mesh.particle_velocity_constraints = pcs
    return pcs


@pytest.mark.parametrize("kw", [dict(), dict(velocity_update=True)])
@pytest.mark.parametrize("scheme", ["usf", "usl"])
def test_particle_constraints_match_oracle(built, scheme, kw):
    steps = 40
    gs, g, info = workloads.plain_small(D, sim_steps=steps, **kw)
    os_, _, _ = workloads.plain_small(O, sim_steps=steps, **kw)
    gs.scheme = scheme
    os_.mpm_scheme = (O.USF if scheme == "usf" else O.USL)(os_.mesh, os_.dt, os_.velocity_update)
    n = info["np"]
    constrained(D, gs, n)
    constrained(O, os_, n)
    sim = gs.simulation(g, reinit=True)
    gs._upload(sim)
    sim.initialize()
    p = os_.mesh.particles[0]
    for i in range(steps):
        sim.step(1)
        os_.step(i, g, reinit=True)
        v = sim.read("velocity")
        assert np.all(v[::7, 0] == np.float32(0.02)) and np.all(v[::5, 1] == np.float32(-0.01))
        assert rel(v, p.velocity.reshape(-1, 2)) <= 1e-5, i
        assert rel(sim.read("loc"), p.loc.reshape(-1, 2)) <= 1e-5, i
        assert close_stress(sim.read("stress"), p.stress.reshape(-1, 6)), i


def test_particle_constraints_line_bitwise(built):
    gs, g = L.bar(D, sim_steps=30)
    os_, _ = L.bar(O, sim_steps=30)
    for s in (gs, os_):
        api = D if s is gs else O
        s.mesh.particle_velocity_constraints = [
            api.ParticleVelocityConstraint(pset=0, pids=np.array([0, 3, 9]), dir=0, velocity=0.01)]
    a = gs.solve_jit(g)
    b = os_.solve_jit(g)
    for k in ("loc", "velocity", "stress"):
        assert np.array_equal(np.asarray(a[k]), np.asarray(b[k])), k


def test_particle_constraints_in_a_batch_and_clearing(built):
    specs = workloads.batch_specs(nsims=2, seed=3, sides=(12, 30))
    sims = []
    for sp in specs:
        solver, g, info = workloads.batch_member(D, sp, sim_steps=20)
        sim = solver.simulation(g, reinit=True)
        solver._upload(sim)
        sim.initialize()
        sims.append(sim)
    n0 = sims[0].n
    ids = np.arange(0, n0, 3)
    sims[0].set_particle_velocity_constraints(ids, np.zeros(ids.size), np.full(ids.size, 0.005))
    batch = D.Batch(sims)
    batch.set_block_steps(10)
    batch.step(20)
    got = sims[0].read("velocity")
    assert np.all(got[::3, 0] == np.float32(0.005))
    solver, g, info = workloads.batch_member(D, specs[0], sim_steps=20)
    alone = solver.simulation(g, reinit=True)
    solver._upload(alone)
    alone.initialize()
    alone.set_particle_velocity_constraints(ids, np.zeros(ids.size), np.full(ids.size, 0.005))
    alone.set_block_steps(10)
    alone.step(20)
    assert np.array_equal(alone.read("velocity"), got)
    assert np.array_equal(alone.read("loc"), sims[0].read("loc"))
    # a constrained run can be recorded and differentiated; clearing the
    # constraints restores the plain step
    alone.record(5, 5)
    seed = np.ones((alone.n, 2), np.float32)
    g1 = alone.adjoint(seed)
    assert all(np.isfinite(v).all() for v in g1.values())
    alone.set_particle_velocity_constraints([], [], [])
    alone.record(5, 5)
    batch.close()
