"""The 1-D step (Linear1D, csrc/mpm_line.cu) against the oracle.

The 1-D kernels add every nodal sum in the reference's scatter order, so the
GPU reproduces the float32 oracle bit for bit; the tolerance checks (1e-5 per
step, as for 2-D) come first so that a failure says how far off it is."""
import numpy as np
import pytest

import diffmpm_gb300 as D
from oracle import mpm_oracle as O
import line_cases as L

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)


CASES = [dict(scheme="usf"), dict(scheme="usl"), dict(scheme="usf", velocity_update=True),
         dict(scheme="usl", material="simple"), dict(scheme="usf", material="simple", nx=7, ppe=1)]


@pytest.mark.parametrize("case", CASES, ids=lambda c: "-".join(f"{k}={v}" for k, v in c.items()))
def test_line_solve_jit_matches_oracle(built, case):
    gs, g = L.bar(D, **case)
    os_, _ = L.bar(O, **case)
    got = gs.solve_jit(g)
    ref = os_.solve_jit(g)
    for k in ("loc", "velocity", "stress", "strain"):
        a, b = np.asarray(got[k]), np.asarray(ref[k])
        assert a.shape == b.shape, k
        assert rel(a, b) <= 1e-5, (k, rel(a, b))
        assert np.array_equal(a, b), (k, rel(a, b))


def test_line_solve_semantics_and_nodes(built):
    """solve (no per-step volume reset) per step, with the nodal state."""
    gs, g = L.bar(D, sim_steps=30)
    os_, _ = L.bar(O, sim_steps=30)
    sim = gs.simulation(g, reinit=False)
    gs._upload(sim)
    sim.initialize()
    p = os_.mesh.particles[0]
    nodes = os_.mesh.elements.nodes
    for i in range(30):
        sim.step(1)
        os_.step(i, g, reinit=False)
        assert np.array_equal(sim.read("loc").reshape(-1), p.loc.reshape(-1)), i
        assert np.array_equal(sim.read("velocity").reshape(-1), p.velocity.reshape(-1)), i
        assert np.array_equal(sim.read("stress"), p.stress.reshape(-1, 6)), i
        assert np.array_equal(sim.read("volume"), p.volume.reshape(-1)), i
        assert np.array_equal(sim.read_nodal("mass"), nodes.mass.reshape(-1)), i
        assert np.array_equal(sim.read_nodal("velocity").reshape(-1), nodes.velocity.reshape(-1)), i
        assert np.array_equal(sim.read_nodal("acceleration").reshape(-1),
                              nodes.acceleration.reshape(-1)), i


def test_line_setup_matches_oracle(built):
    gs, g = L.bar(D, nx=9, ppe=2)
    os_, _ = L.bar(O, nx=9, ppe=2)
    pg, po = gs.mesh.particles[0], os_.mesh.particles[0]
    assert np.array_equal(pg.element_ids, po.element_ids)
    assert np.array_equal(pg.volume.reshape(-1), po.volume.reshape(-1))
    assert np.array_equal(pg.mass.reshape(-1), po.mass.reshape(-1))


def test_line_leaving_the_mesh_raises(built):
    gs, g = L.bar(D, nx=8, ppe=1, sim_steps=5)
    gs.mesh.particles[0].velocity[:] = 400.0
    with pytest.raises(D.OutOfMeshError):
        gs.solve_jit(g)


def test_line_unsupported_parts(built):
    gs, g = L.bar(D, sim_steps=3)
    sim = gs.simulation(g, reinit=True)
    gs._upload(sim)
    sim.initialize()
    with pytest.raises(D.MpmError):
        D.Batch([sim])
    with pytest.raises(D.MpmError):
        sim.run_phase("nodal_kinematics")


def test_line_adjoint_refusals(built):
    """The 1-D adjoint needs a recording that is still current."""
    gs, g = L.bar(D, sim_steps=3)
    sim = gs.simulation(g, reinit=True)
    gs._upload(sim)
    sim.initialize()
    seed = np.ones((sim.n, 1), np.float32)
    with pytest.raises(D.MpmError):
        sim.adjoint(seed)            # nothing recorded
    sim.record(3)
    sim.step(1)                      # the recorded run is overwritten
    with pytest.raises(D.MpmError):
        sim.adjoint(seed)
    sim.close()
