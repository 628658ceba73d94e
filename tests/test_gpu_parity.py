"""Parity of the CUDA step with the oracle, through the C ABI.

Tolerances (normwise relative error ||gpu - oracle|| / ||oracle||, float32 on
both sides): 1e-5 per step on nodal and particle fields, 1e-4 on positions
after a full run.  The goldens of the reference's benchmark tests are checked
at the reference's own decimals.

A field whose exact value is zero (the stress of a block in free fall) holds
only float32 round-off in both implementations, and the two round-offs differ
because the nodal sums are accumulated in different orders.  For such a field
(stress, strain and the centroid volumetric strain only) the check may pass
against the float64 oracle instead: the GPU must be as close to float64 as the
float32 restatement of the reference is (within 3x), which is the "error vs
FP64" criterion.  Every field that passes that way is listed at the end of the
run; any other field must meet the tolerance itself.
"""
import numpy as np
import pytest

import diffmpm_gb300 as D
from diffmpm_gb300 import workloads
from oracle import mpm_oracle as O
import decks

pytestmark = pytest.mark.gpu

STEP_TOL = 1e-5
RUN_TOL = 1e-4


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def oracle_fields(solver):
    p = solver.mesh.particles[0]
    return {"loc": p.loc.reshape(-1, 2), "velocity": p.velocity.reshape(-1, 2),
            "stress": p.stress.reshape(-1, 6), "strain": p.strain.reshape(-1, 6),
            "density": p.density.reshape(-1),
            "volumetric_strain_centroid": p.volumetric_strain_centroid.reshape(-1)}


def gpu_fields(sim):
    return {k: sim.read(k) for k in ("loc", "velocity", "stress", "strain", "density",
                                      "volumetric_strain_centroid")}


def start_pair(builder, reinit=True, **kw):
    """(gpu Simulation initialised, oracle solver, gravity) for the same input;
    the float64 oracle is attached as ``oracle.f64``."""
    gs, g, info = builder(D, **kw)
    os_, _, _ = builder(O, **kw)
    os_.f64, _, _ = builder(O, dtype=np.float64, **kw)
    sim = gs.simulation(g, reinit=reinit)
    gs._upload(sim)
    sim.initialize()
    return sim, os_, g


# Absolute round-off floors per particle for fields whose exact value can be
# zero: 1 mPa of stress and a strain of 1e-9 (every configuration here has
# E >= 1e3 Pa, so these are far below any stress or strain it develops).
FLOOR = {"stress": 1e-3, "strain": 1e-9, "volumetric_strain_centroid": 1e-9}


# Every check that passed through the round-off floor or the float64
# criterion instead of the plain tolerance: (check, rel. error against the
# float32 oracle, how it passed); printed at the end of the run.
FALLBACKS = []


def close(name, gpu, f32, f64, tol, field=None):
    """``gpu`` matches the float32 oracle within ``tol``.  Only for the fields
    of ``FLOOR``, whose exact value can be zero, a miss may instead pass by
    differing from the float32 oracle by less than the round-off floor, or by
    being as close to float64 as the float32 oracle is (within 3x); each such
    pass is recorded in ``FALLBACKS``."""
    e = rel(gpu, f32)
    if e <= tol:
        return e
    floor = FLOOR.get(field)
    assert floor is not None, (name, e, f"misses {tol:g} on a field that is not zero-valued")
    diff = np.linalg.norm(np.asarray(gpu, np.float64) - np.asarray(f32, np.float64))
    if diff <= floor * np.sqrt(np.size(gpu)):
        FALLBACKS.append((name, e, f"within the round-off floor {floor:g}"))
        return e
    e_gpu, e_ref = rel(gpu, f64), rel(f32, f64)
    assert e_gpu <= max(3.0 * e_ref, tol), (name, e, e_gpu, e_ref)
    FALLBACKS.append((name, e, f"float64 criterion: GPU {e_gpu:.2e} vs float32 oracle {e_ref:.2e}"))
    return e


def nodal_fields(osv, sim):
    nodes = osv.mesh.elements.nodes
    return {k: getattr(nodes, k).reshape(sim.read_nodal(k).shape)
            for k in ("mass", "velocity", "acceleration")}


def step_and_compare(sim, osv, g, nsteps, reinit=True, every=1, tol=STEP_TOL, nodal=True):
    worst = {}
    for i in range(nsteps):
        sim.step(1)
        osv.step(i, g, reinit=reinit)
        osv.f64.step(i, g, reinit=reinit)
        if (i + 1) % every:
            continue
        a, b, c = gpu_fields(sim), oracle_fields(osv), oracle_fields(osv.f64)
        for k in a:
            worst[k] = max(worst.get(k, 0.0), close((i, k), a[k], b[k], c[k], tol, k))
        if nodal:
            b, c = nodal_fields(osv, sim), nodal_fields(osv.f64, sim)
            for k in b:
                worst["node_" + k] = max(worst.get("node_" + k, 0.0),
                                         close((i, "node " + k), sim.read_nodal(k), b[k], c[k], tol))
    return worst


@pytest.mark.parametrize("name", ["uniaxial_stress", "uniaxial_nodal_forces",
                                  "uniaxial_particle_traction"])
def test_benchmark_goldens(built, name):
    deck = decks.load_deck(name)
    stress = {}
    solver, g = decks.build(D, deck, writer_func=lambda a, t, **kw: stress.__setitem__(a[1], a[0]["stress"]))
    solver.solve_jit(g)
    decks.check_goldens(deck, stress)
    # and against the oracle at every golden step
    ref = {}
    osv, _ = decks.build(O, deck, writer_func=lambda a, i: ref.__setitem__(i, a["stress"]))
    osv.solve_jit(g)
    for gg in deck["goldens"]:
        i = gg["file_index"]
        assert rel(stress[i], ref[i]) <= RUN_TOL, (i, rel(stress[i], ref[i]))


def test_plain_small_per_step(built):
    sim, osv, g = start_pair(workloads.plain_small, sim_steps=60)
    step_and_compare(sim, osv, g, 60)


def test_plain_small_full_run(built):
    gs, g, _ = workloads.plain_small(D)
    os_, _, _ = workloads.plain_small(O)
    o64, _, _ = workloads.plain_small(O, dtype=np.float64)
    a = gs.solve_jit(g)
    b = os_.solve_jit(g)
    c = o64.solve_jit(g)
    assert rel(a["loc"], b["loc"]) <= RUN_TOL
    for k in ("velocity", "stress", "strain"):
        close(k, a[k], b[k], c[k], RUN_TOL, k)


@pytest.mark.parametrize("scheme", ["usf", "usl"])
def test_scaleup_reduced(built, scheme):
    sim, osv, g = start_pair(workloads.plain_scaleup, n=48, scheme=scheme, sim_steps=12)
    step_and_compare(sim, osv, g, 12, every=3)


def test_mixed_newtonian_reduced(built):
    sim, osv, g = start_pair(workloads.mixed_large, n=48, sim_steps=12)
    step_and_compare(sim, osv, g, 12, every=3)


def test_velocity_update_true(built):
    sim, osv, g = start_pair(workloads.plain_small, sim_steps=30, velocity_update=True)
    step_and_compare(sim, osv, g, 30, every=5)


def test_solve_semantics_no_reinit(built):
    sim, osv, g = start_pair(workloads.plain_small, reinit=False, sim_steps=40)
    step_and_compare(sim, osv, g, 40, reinit=False, every=4)


def test_phases_match_oracle(built):
    """Nodal kinematics, forces + nodal update and G2P, one phase at a time."""
    sim, osv, g = start_pair(workloads.plain_scaleup, n=32, scheme="usf", sim_steps=3)
    nodes = osv.mesh.elements.nodes
    for i in range(3):
        osv._setup_volume()
        s = osv.mpm_scheme
        sim.run_phase("nodal_kinematics")
        s.compute_nodal_kinematics()
        assert rel(sim.read_nodal("mass"), nodes.mass.reshape(-1)) <= STEP_TOL
        s.precompute_stress_strain()
        s.compute_forces(g, i)
        sim.run_phase("forces")
        s.compute_particle_kinematics()
        assert rel(sim.read_nodal("velocity"), nodes.velocity.reshape(-1, 2)) <= STEP_TOL
        assert rel(sim.read_nodal("acceleration"), nodes.acceleration.reshape(-1, 2)) <= STEP_TOL
        sim.run_phase("particle_kinematics")
        s.postcompute_stress_strain()
        a, b = gpu_fields(sim), oracle_fields(osv)
        for k in a:
            assert rel(a[k], b[k]) <= STEP_TOL, (i, k)


def test_deterministic(built):
    outs = []
    for _ in range(2):
        gs, g, _ = workloads.plain_scaleup(D, n=64, sim_steps=25)
        outs.append(gs.solve_jit(g))
    for k in outs[0]:
        assert np.array_equal(outs[0][k], outs[1][k]), k


def fast_builder(api, v=(0.6, 0.25), steps=60, **kw):
    """plain_small with a uniform initial velocity fast enough to cross cells."""
    return workloads.plain_small(api, sim_steps=steps, dt=2e-3, velocity=v, **kw)


def test_cell_crossing_resorts(built):
    """Particles crossing cells trigger re-sorts; results still match."""
    sim, osv, g = start_pair(fast_builder, steps=60)
    sim.set_block_steps(10)
    step_and_compare(sim, osv, g, 60, every=10)
    c = sim.counters()
    assert c["resorts"] >= 2


def test_drift_rollback(built):
    """A block in which a particle drifts two cells from its sort-cell is rolled
    back and replayed step by step; results still match the oracle."""
    # 0.3 cells per step: within 5 steps half the particles cross two cell edges
    gs, g, _ = fast_builder(D, v=(15.0, 0.0), steps=5)
    os_, _, _ = fast_builder(O, v=(15.0, 0.0), steps=5)
    sim = gs.simulation(g)
    gs._upload(sim)
    sim.initialize()
    sim.set_block_steps(5)
    sim.step(5)
    for i in range(5):
        os_.step(i, g)
    o64, _, _ = fast_builder(O, v=(15.0, 0.0), steps=5, dtype=np.float64)
    for i in range(5):
        o64.step(i, g)
    assert sim.counters()["rollbacks"] >= 1
    a, b, c = gpu_fields(sim), oracle_fields(os_), oracle_fields(o64)
    for k in a:
        close(k, a[k], b[k], c[k], STEP_TOL, k)


def test_cfl_violation_raises(built):
    """A particle crossing two cells in one step is reported, not mis-summed."""
    gs, g, _ = fast_builder(D, v=(120.0, 0.0), steps=3)
    sim = gs.simulation(g)
    gs._upload(sim)
    sim.initialize()
    with pytest.raises(D.MpmError) as e:
        sim.step(3)
    assert e.value.code in (3, 4)


def test_out_of_mesh_raises(built):
    gs, g, _ = workloads.plain_small(D, sim_steps=2)
    sim = gs.simulation(g)
    gs._upload(sim)
    loc = sim.read("loc")
    loc[0] = [1.5, 0.5]
    sim.write("loc", loc)
    with pytest.raises(D.OutOfMeshError):
        sim.initialize()


def test_long_block_drift_is_rolled_back(built):
    """In a long step block a particle can drift two cells from its sort-cell;
    the sums of the rest of the block are then wrong and may throw particles
    out of the mesh.  The block must be rolled back and replayed (not reported
    as out-of-mesh), and the run must match the oracle (a soft block on a 1 m
    domain, 100-step blocks, 200 steps)."""
    spec = workloads.batch_specs(domain=1.0, velocity_update=True)[332]
    gs, g, _ = workloads.batch_member(D, spec, sim_steps=200)
    sim = gs.simulation(g)
    gs._upload(sim)
    sim.initialize()
    sim.set_block_steps(100)
    sim.step(200)
    assert sim.counters()["rollbacks"] >= 1
    os_, og, _ = workloads.batch_member(O, spec, sim_steps=200)
    for i in range(200):
        os_.step(i, og)
    assert rel(sim.read("loc"), os_.mesh.particles[0].loc.reshape(-1, 2)) < RUN_TOL
