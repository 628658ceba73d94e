"""Properties checked at the benchmark configurations' full sizes, where the
oracle is too slow: bitwise reproducibility of the 1024^2 scale-up, a batch
of one equal to the simulation run alone, the 4096^2 elastic + Newtonian run
reproducible and unchanged by where its step blocks split, and the adjoint of
the 256^2 differentiation run (2000 steps, checkpoints every 100) linear in
its seed."""
import numpy as np
import pytest

import diffmpm_gb300 as D
from diffmpm_gb300 import workloads

pytestmark = pytest.mark.gpu

FIELDS = ("loc", "velocity", "stress", "strain", "density")


def scaleup_sim(steps):
    solver, g, info = workloads.plain_scaleup(D, n=1024, sim_steps=steps)
    sim = solver.simulation(g, reinit=True)
    solver._upload(sim)
    sim.initialize()
    sim.set_block_steps(10)
    return solver, sim, info


def test_scaleup_full_size_reproducible_and_batch_of_one(built):
    steps = 30
    solver, sim, info = scaleup_sim(steps)
    assert info["np"] == 2097152
    sim.step(steps)
    first = {k: sim.read(k).copy() for k in FIELDS}
    solver._upload(sim)
    sim.initialize()
    sim.step(steps)
    for k in FIELDS:
        assert np.array_equal(sim.read(k), first[k]), k
    assert np.isfinite(first["stress"]).all()
    solver._upload(sim)
    sim.initialize()
    b = D.Batch([sim])
    b.set_block_steps(10)
    b.step(steps)
    for k in FIELDS:
        assert np.array_equal(sim.read(k), first[k]), ("batch", k)
    b.close()
    sim.close()


def test_mixed_large_full_size_reproducible_and_split_blocks_agree(built):
    """4096^2 mesh, 16,777,216 particles in a LinearElastic and a Newtonian
    block, USL, 200 steps of 2e-7 s: two runs agree bitwise, a run advanced as
    120 + 80 steps in blocks of 40 equals one advanced as 200 in blocks of 100,
    and every particle stays finite and inside the mesh."""
    steps = 200
    solver, g, info = workloads.mixed_large(D, sim_steps=steps)
    assert info["np"] == 16777216
    sim = solver.simulation(g, reinit=True)
    fields = ("loc", "velocity", "stress", "density")

    def run(block, parts):
        solver._upload(sim)
        sim.initialize()
        sim.set_block_steps(block)
        for k in parts:
            sim.step(k)
        return {k: sim.read(k).copy() for k in fields}

    first = run(100, (steps,))
    for k in fields:
        assert np.isfinite(first[k]).all(), k
    loc = first["loc"].reshape(-1, 2)
    assert loc.min() >= 0.0 and loc.max() < 1.0
    again = run(100, (steps,))
    split = run(40, (120, 80))
    for k in fields:
        assert np.array_equal(again[k], first[k]), k
        assert np.array_equal(split[k], first[k]), ("split", k)
    sim.close()


def test_differentiation_full_size_adjoint_is_linear_in_the_seed(built):
    solver, g, info = workloads.differentiation(D)
    assert info["np"] == 125664
    sim = solver.simulation(g, reinit=True)
    solver._upload(sim)
    sim.initialize()
    sim.record(2000, 100)
    rng = np.random.Generator(np.random.PCG64(3))
    s1 = rng.normal(size=(info["np"], 2)).astype(np.float32)
    s2 = rng.normal(size=(info["np"], 2)).astype(np.float32)
    g1 = sim.adjoint(s1)
    g1b = sim.adjoint(s1)
    g2x = sim.adjoint(2.0 * s1)          # scaling by 2 is exact in float32
    g12 = sim.adjoint(s1 + s2)
    g2 = sim.adjoint(s2)
    for k in g1:
        assert np.isfinite(g1[k]).all(), k
        assert np.array_equal(g1[k], g1b[k]), k                      # repeatable
        hom = np.linalg.norm(g2x[k] - 2.0 * g1[k].astype(np.float64)) / max(
            np.linalg.norm(2.0 * g1[k].astype(np.float64)), 1e-30)
        assert hom < 1e-6, (k, hom)     # homogeneous (exact unless a product underflows)
        lin = g1[k].astype(np.float64) + g2[k]
        err = np.linalg.norm(g12[k] - lin) / max(np.linalg.norm(lin), 1e-30)
        assert err < 1e-4, (k, err)                                   # additive up to rounding
    sim.close()
