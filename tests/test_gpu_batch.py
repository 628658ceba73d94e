"""Batches of independent simulations (mpm_batch_*) against single runs.

A batch runs the same tile kernels over the tiles of all its simulations, so
every member must end bit for bit where the same simulation run alone (with
the same step-block size, hence the same re-sort schedule) ends, and within
the parity tolerances of the oracle.
"""
import numpy as np
import pytest

import diffmpm_gb300 as D
from diffmpm_gb300 import workloads
from oracle import mpm_oracle as O

pytestmark = pytest.mark.gpu

FIELDS = ("loc", "velocity", "stress", "strain", "density")


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def small_specs(k=5, seed=3):
    return workloads.batch_specs(nsims=k, seed=seed, sides=(12, 40))


def member_sim(spec, steps):
    solver, g, info = workloads.batch_member(D, spec, sim_steps=steps)
    sim = solver.simulation(g, reinit=True)
    solver._upload(sim)
    sim.initialize()
    return solver, sim, g


def state(sim):
    return {k: sim.read(k).copy() for k in FIELDS}


def test_batch_equals_single_runs(built):
    specs = small_specs()
    steps = 60
    members = [member_sim(sp, steps) for sp in specs]
    batch = D.Batch([m[1] for m in members])
    n, ntiles = batch.size()
    assert n == len(specs) and ntiles > n
    batch.set_block_steps(20)
    batch.step(steps)
    for sp in specs:
        _, alone, _ = member_sim(sp, steps)
        alone.set_block_steps(20)
        alone.step(steps)
        ref = state(alone)
        got = state(members[specs.index(sp)][1])
        for k in FIELDS:
            assert np.array_equal(got[k], ref[k]), (sp["side"], k)
    for _, sim, _ in members:
        assert sim.step_index == steps


def test_batch_member_matches_oracle(built):
    spec = small_specs(k=1, seed=11)[0]
    steps = 40
    solver, sim, g = member_sim(spec, steps)
    other = member_sim(small_specs(k=2, seed=12)[1], steps)
    batch = D.Batch([sim, other[1]])
    batch.step(steps)
    o, og, _ = workloads.batch_member(O, spec, sim_steps=steps)
    exp = o.solve_jit(og)
    assert rel(sim.read("loc"), exp["loc"].reshape(-1, 2)) < 1e-4
    assert rel(sim.read("velocity"), exp["velocity"].reshape(-1, 2)) < 1e-4


def test_autotune_leaves_state_unchanged(built):
    specs = small_specs(k=4, seed=7)
    members = [member_sim(sp, 30) for sp in specs]
    batch = D.Batch([m[1] for m in members])
    batch.step(5)
    before = [state(m[1]) for m in members]
    steps_before = [m[1].step_index for m in members]
    t = batch.autotune(trial_steps=30, cache=False)
    assert t["block_steps"] >= 1 and t["resort_every"] in (1, 2, 4) and t["ms_per_step"] > 0
    assert t["nk_ctas"] in (2, 3) and t["g2p_ctas"] in (2, 3) and not t["from_cache"]
    assert batch.tuning()["block_steps"] == t["block_steps"]
    for m, st, sb in zip(members, before, steps_before):
        assert m[1].step_index == sb
        now = state(m[1])
        for k in FIELDS:
            assert np.array_equal(now[k], st[k]), k


def test_batch_rollback_matches_single(built):
    """A member whose particles drift two cells inside a block is rolled back
    and replayed alone, exactly as a single run does."""
    # 0.3 cells per step: within 5 steps particles cross two cell edges
    specs = small_specs(k=3, seed=9)
    fast = workloads.plain_small(D, sim_steps=5, dt=2e-3, velocity=(15.0, 0.0))
    members = [member_sim(sp, 5) for sp in specs]
    gs, g, _ = fast
    fsim = gs.simulation(g, reinit=True)
    gs._upload(fsim)
    fsim.initialize()
    batch = D.Batch([members[0][1], fsim, members[1][1], members[2][1]])
    batch.set_block_steps(5)
    batch.step(5)
    assert fsim.counters()["rollbacks"] >= 1
    alone_solver, ag, _ = workloads.plain_small(D, sim_steps=5, dt=2e-3, velocity=(15.0, 0.0))
    alone = alone_solver.simulation(ag, reinit=True)
    alone_solver._upload(alone)
    alone.initialize()
    alone.set_block_steps(5)
    alone.step(5)
    for k in FIELDS:
        assert np.array_equal(fsim.read(k), alone.read(k)), k


def test_batch_rejects_mixed_configurations(built):
    a = member_sim(small_specs(k=1)[0], 5)[1]
    s2, g2, _ = workloads.plain_scaleup(D, n=16, scheme="usl", sim_steps=2)
    b = s2.simulation(g2, reinit=True)
    s2._upload(b)
    b.initialize()
    with pytest.raises(D.MpmError) as e:
        D.Batch([a, b])
    assert e.value.code == 5
    with pytest.raises(D.MpmError):
        D.Batch([a, a])


@pytest.mark.parametrize("scheme", ["usf", "usl"])
@pytest.mark.parametrize("reinit", [True, False])
def test_batch_variants_equal_single_runs(built, scheme, reinit):
    """Every batched kernel variant (scheme x volume set-up x forces path)
    gives each member the bits of its single run."""
    specs = small_specs(k=3, seed=21)
    steps = 30

    def make(sp):
        solver, g, _ = workloads.batch_member(D, sp, sim_steps=steps)
        solver.scheme = scheme
        sim = solver.simulation(g, reinit=reinit)
        solver._upload(sim)
        sim.initialize()
        sim.set_block_steps(10)
        return sim

    alone = []
    for sp in specs:
        sim = make(sp)
        sim.step(steps)
        alone.append(state(sim))
    for lpc in (0, 1, 2):
        members = [make(sp) for sp in specs]
        batch = D.Batch(members)
        batch.set_tuning(block_steps=10, resort_every=1, forces_lpc=lpc)
        batch.step(steps)
        for sp, sim, ref in zip(specs, members, alone):
            for k in FIELDS:
                assert np.array_equal(sim.read(k), ref[k]), (lpc, sp["side"], k)
        batch.close()


def test_batch_with_tractions_equals_single_runs(built):
    """The traction variant of the batched forces kernel, on the particle
    traction benchmark deck (two copies with different Young's moduli)."""
    import decks
    deck = decks.load_deck("uniaxial_particle_traction")
    steps = 200

    def make(E):
        d = dict(deck, materials=[dict(deck["materials"][0], youngs_modulus=E)])
        solver, g = decks.build(D, d, sim_steps=steps)
        sim = solver.simulation(g, reinit=True)
        solver._upload(sim)
        sim.initialize()
        sim.set_block_steps(25)
        return sim

    members = [make(1e6), make(2e6)]
    batch = D.Batch(members)
    batch.set_block_steps(25)
    batch.step(steps)
    for E, sim in zip((1e6, 2e6), members):
        alone = make(E)
        alone.step(steps)
        for k in FIELDS:
            assert np.array_equal(sim.read(k), alone.read(k)), (E, k)
    batch.close()


def test_batch_state_transfers_and_restart(built):
    """Whole-batch writes read back bit for bit, and a restart from the
    written initial states runs like freshly uploaded simulations."""
    specs = small_specs(k=3, seed=31)
    steps = 40
    members = [member_sim(sp, steps) for sp in specs]
    sims = [m[1] for m in members]
    batch = D.Batch(sims)
    batch.set_block_steps(10)
    batch.step(15)
    # write the members' initial states back (one array per field)
    init = {}
    for k, attr in (("loc", "loc"), ("velocity", "velocity"), ("stress", "stress"),
                    ("strain", "strain"), ("density", "density"),
                    ("volumetric_strain_centroid", "volumetric_strain_centroid")):
        init[k] = np.concatenate([np.asarray(getattr(m[0].mesh.particles[0], attr), np.float32)
                                  .reshape(-1) for m in members])
        batch.write(k, init[k])
        assert np.array_equal(batch.read(k), init[k]), k
    per = batch.split("loc", batch.read("loc"))
    for p, (solver, sim, g) in zip(per, members):
        assert np.array_equal(p, sim.read("loc"))
    batch.write_nodal("velocity", [np.zeros((s.nnodes, 2), np.float32) for s in sims])
    batch.restart()
    assert all(s.step_index == 0 for s in sims)
    batch.step(steps)
    for sp, sim in zip(specs, sims):
        _, alone, _ = member_sim(sp, steps)
        alone.set_block_steps(10)
        alone.step(steps)
        for k in ("loc", "velocity", "stress"):
            assert rel(sim.read(k), alone.read(k)) <= 1e-6, (sp["side"], k)
    with pytest.raises(D.MpmError):
        batch.write("material_id", np.zeros(sum(s.n for s in sims), np.float32))
    batch.close()


def test_autotune_result_is_cached_and_read_back(built, tmp_path):
    """The tuning chosen for a configuration is stored in the cache under
    (GPU name, configuration hash) and the next autotune of the same
    configuration reads it back without timing and applies it; another
    configuration misses the cache."""
    import json
    cache = tmp_path / "tuning.json"
    specs = small_specs(k=3, seed=11)
    a = D.Batch([member_sim(sp, 30)[1] for sp in specs])
    t1 = a.autotune(trial_steps=20, cache=cache)
    assert not t1["from_cache"]
    stored = json.loads(cache.read_text())
    assert t1["key"] in stored and t1["key"].startswith(D.engine.device_name())
    b = D.Batch([member_sim(sp, 30)[1] for sp in specs])
    t2 = b.autotune(trial_steps=20, cache=cache)
    assert t2["from_cache"] and t2["key"] == t1["key"]
    for k in ("block_steps", "resort_every", "nk_ctas", "g2p_ctas", "forces_lpc"):
        assert t2[k] == t1[k] and b.tuning()[k] == t1[k], k
    c = D.Batch([member_sim(sp, 30)[1] for sp in small_specs(k=2, seed=12)])
    t3 = c.autotune(trial_steps=20, cache=cache)
    assert not t3["from_cache"] and t3["key"] != t1["key"]
    assert len(json.loads(cache.read_text())) == 2


def test_kernel_builds_and_resort_cadence_keep_results(built):
    """Every kernel build gives the same bits; a re-sort every second block
    stays within the parity tolerance of the oracle."""
    spec = small_specs(k=1, seed=13)[0]
    ref = None
    for nk, g2p, lpc in ((3, 3, 0), (2, 2, 1), (3, 2, 2), (2, 3, 0)):
        _, sim, _ = member_sim(spec, 40)
        b = D.Batch([sim])
        b.set_tuning(block_steps=10, resort_every=1, nk_ctas=nk, g2p_ctas=g2p, forces_lpc=lpc)
        b.step(40)
        got = state(sim)
        if ref is None:
            ref = got
        for k in FIELDS:
            assert np.array_equal(got[k], ref[k]), (nk, g2p, lpc, k)
    _, sim, _ = member_sim(spec, 40)
    b = D.Batch([sim])
    b.set_tuning(block_steps=10, resort_every=2)
    b.step(40)
    o, og, _ = workloads.batch_member(O, spec, sim_steps=40)
    exp = o.solve_jit(og)
    assert rel(sim.read("loc"), exp["loc"].reshape(-1, 2)) < 1e-4
    assert rel(sim.read("velocity"), exp["velocity"].reshape(-1, 2)) < 1e-4


@pytest.mark.parametrize("builder,kw,reinit", [
    (workloads.plain_scaleup, dict(n=64, scheme="usf"), True),
    (workloads.plain_scaleup, dict(n=64, scheme="usl"), True),
    (workloads.mixed_large, dict(n=48), True),
    (workloads.plain_scaleup, dict(n=64, scheme="usf"), False),
    (workloads.plain_scaleup, dict(n=64, scheme="usl"), False),
])
def test_forces_paths_give_the_same_bits(built, builder, kw, reinit):
    """The forces kernel's three fast paths (particle per lane with row
    slots, lane per cell in global memory, particle per lane on a staged
    row) add every cell's contributions in the same order: a single
    simulation ends bit for bit in the same state with each, with the
    per-step volume set-up and under solve semantics (persistent volume)."""
    out = []
    for lpc in (0, 1, 2):
        s, g, _ = builder(D, sim_steps=30, **kw)
        sim = s.simulation(g, reinit=reinit)
        s._upload(sim)
        sim.initialize()
        sim.set_kernel_variant(3, 2, lpc)
        sim.set_block_steps(10)
        sim.step(30)
        out.append(state(sim))
        sim.close()
    for o in out[1:]:
        for k in FIELDS:
            assert np.array_equal(out[0][k], o[k]), k
