"""The oracle's definitions of the build's extensions (no reference to pin
them): particle velocity constraints and the 1-D step."""
import numpy as np

from diffmpm_gb300 import workloads
from oracle import mpm_oracle as O
import line_cases as L


def test_particle_velocity_constraints_set_velocity_and_momentum():
    solver, g, info = workloads.plain_small(O, sim_steps=3)
    n = info["np"]
    solver.mesh.particle_velocity_constraints = [
        O.ParticleVelocityConstraint(pset=0, pids=np.arange(0, n, 4), dir=1, velocity=0.25),
        O.ParticleVelocityConstraint(pset=0, pids=np.arange(0, n, 8), dir=1, velocity=-0.5)]
    free, _, _ = workloads.plain_small(O, sim_steps=3)
    for i in range(3):
        solver.step(i, g)
        free.step(i, g)
    p = solver.mesh.particles[0]
    v = p.velocity.reshape(-1, 2)
    assert np.all(v[::8, 1] == np.float32(-0.5))                     # later entries win
    assert np.all(v[4::8, 1] == np.float32(0.25))
    assert np.array_equal(p.momentum, p.mass * p.velocity)
    # positions still move with the nodal velocity of the first step
    x1 = free.mesh.particles[0].loc.reshape(-1, 2)
    assert not np.array_equal(v[:, 1], free.mesh.particles[0].velocity.reshape(-1, 2)[:, 1])
    assert x1.shape == p.loc.reshape(-1, 2).shape


def test_line_bar_runs_and_conserves_sanity():
    solver, g = L.bar(O, sim_steps=20, gravity=0.0)
    r = solver.solve_jit(g)
    assert np.isfinite(r["stress"]).all() and np.isfinite(r["loc"]).all()
    # 1-D: only the xx strain component moves (the build's 1-D strain rate)
    assert np.all(r["strain"][:, 1:] == 0.0) and np.any(r["strain"][:, 0] != 0.0)
