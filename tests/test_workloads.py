"""The benchmark workload builders (diffmpm_gb300/workloads.py) on the CPU,
through the oracle's classes: particle counts, material split, seeded
velocities and placement, at sizes the oracle builds in a second, plus the
full-size particle counts the benchmark reports."""
import numpy as np

from diffmpm_gb300 import workloads
from oracle import mpm_oracle as O


def _particles(solver):
    return solver.mesh.particles[0]


def test_mixed_large_blocks_and_seeded_velocities():
    for n in (64, 128):
        solver, g, info = workloads.mixed_large(O, n=n, sim_steps=1)
        ps = _particles(solver)
        loc = np.asarray(ps.loc).reshape(-1, 2)
        mid = np.asarray(ps.material_ids)
        # two blocks of n/4 x n/2 cells, 4 Gauss points per cell: n^2 particles
        # (16,777,216 at the benchmark's 4096^2), half of them in each material
        assert info["np"] == n * n == len(loc)
        assert (mid == 0).sum() == (mid == 1).sum() == n * n // 2
        assert loc[mid == 0, 0].max() < 0.375 <= loc[mid == 1, 0].min()
        assert loc[:, 1].min() > 0.0 and loc[:, 1].max() < 0.5
        v = np.asarray(ps.velocity).reshape(-1, 2)
        assert abs(v.std() - 0.01) < 0.002 and abs(v.mean()) < 0.002
        assert solver.scheme == "usl" and np.allclose(g, [0.0, -9.81])
    again, _, _ = workloads.mixed_large(O, n=64, sim_steps=1)
    first, _, _ = workloads.mixed_large(O, n=64, sim_steps=1)
    assert np.array_equal(np.asarray(_particles(again).velocity),
                          np.asarray(_particles(first).velocity))


def test_scaleup_and_differentiation_counts():
    _, _, info = workloads.plain_scaleup(O, n=64, sim_steps=1)
    assert info["np"] == 64 * 32 * 4          # 2,097,152 at 1024^2
    _, _, info = workloads.differentiation(O, sim_steps=1)
    assert info["np"] == 125664               # 204 x 154 cells x 4 at 256^2
