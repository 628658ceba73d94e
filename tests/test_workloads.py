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


def test_batching_configuration_members():
    """The 512 seeded members of the batching configuration: mesh sides in
    32..256, rectangles of 20-60 % of the domain resting on the bottom inside
    a 5 % wall margin, E log-uniform in [1e5, 1e8], nu in [0.2, 0.35], the
    CFL time step 0.3 h / c_p, and 19,580,520 particles in all (the count the
    benchmark reports); the same seed gives the same members."""
    specs = workloads.batch_specs()
    assert len(specs) == 512
    assert sum(s["np"] for s in specs) == 19_580_520
    for s in specs:
        n = s["side"]
        i0, i1, j0, j1 = s["cells"]
        assert 32 <= n <= 256 and j0 == 0
        margin = int(np.ceil(0.05 * n))
        assert margin <= i0 < i1 <= n - margin and j1 <= n - margin
        assert s["np"] == 4 * (i1 - i0) * (j1 - j0)
        assert 1e5 <= s["E"] <= 1e8 and 0.2 <= s["nu"] <= 0.35
        M = s["E"] * (1 - s["nu"]) / ((1 + s["nu"]) * (1 - 2 * s["nu"]))
        assert np.isclose(s["dt"], 0.3 * (s["domain"] / n) / np.sqrt(M / s["rho"]), rtol=1e-12)
    sides = [s["side"] for s in specs]
    assert min(sides) < 48 and max(sides) > 240
    assert workloads.batch_specs() == specs


def test_batch_member_particles_are_the_specs_gauss_points():
    spec = workloads.batch_specs(nsims=3)[2]
    solver, g, info = workloads.batch_member(O, spec, sim_steps=1)
    loc = np.asarray(_particles(solver).loc).reshape(-1, 2)
    assert info["np"] == spec["np"] == len(loc)
    h = spec["domain"] / spec["side"]
    i0, i1, j0, j1 = spec["cells"]
    cells = np.floor(loc / h).astype(int)
    assert cells[:, 0].min() == i0 and cells[:, 0].max() == i1 - 1
    assert cells[:, 1].min() == j0 and cells[:, 1].max() == j1 - 1
    # 4 Gauss points per cell
    _, counts = np.unique(cells[:, 1] * spec["side"] + cells[:, 0], return_counts=True)
    assert (counts == 4).all()
    assert np.allclose(g, [0.0, -9.81]) and solver.scheme == "usf"
