"""TOML decks end to end on the GPU: ``MPM(deck).solve()`` writes
``results/<title>/particles_<step>.npz`` as the reference does, and the
goldens of the reference's benchmark tests (benchmarks/2d/*/test_benchmark.py)
are checked on those files.  Also the asynchronous output path
(mpm_output_enqueue / mpm_output_wait) against plain reads."""
import os
import subprocess
import sys

import numpy as np
import pytest

import diffmpm_gb300 as D
from diffmpm_gb300 import workloads
from oracle import mpm_oracle as O
import decks
import toml_decks

pytestmark = pytest.mark.gpu

NAMES = ["uniaxial_stress", "uniaxial_nodal_forces", "uniaxial_particle_traction"]


def npz_name(step, nsteps):
    return f"particles_{step:0{len(str(nsteps))}d}.npz"


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)


@pytest.mark.parametrize("name", NAMES)
def test_deck_goldens_from_npz(built, tmp_path, monkeypatch, name):
    deck = decks.load_deck(name)
    toml_decks.write_deck(deck, tmp_path)
    monkeypatch.chdir(tmp_path)
    D.MPM("deck.toml").solve()
    meta, out = deck["meta"], deck["output"]
    folder = tmp_path / out["folder"] / meta["title"]
    want = {npz_name(i, meta["nsteps"]) for i in range(0, meta["nsteps"], out["step_frequency"])}
    assert {p.name for p in folder.iterdir()} == want
    stress = {}
    for g in deck["goldens"]:
        with np.load(folder / npz_name(g["file_index"], meta["nsteps"])) as f:
            assert set(f.files) == {"loc", "velocity", "stress", "strain"}
            np_ = len(deck["particles"][0]["loc"])
            assert f["stress"].shape == (1, np_, 6) and f["loc"].shape == (1, np_, 2)
            stress[g["file_index"]] = f["stress"]
    decks.check_goldens(deck, stress)
    # the same files as the oracle's writer gives, step for step
    ref = {}
    osv, _ = decks.build(O, deck, writer_func=lambda a, i: ref.__setitem__(i, a))
    osv.solve_jit(np.asarray(deck["external_loading"]["gravity"], float))
    # (positions and stresses, as the golden checks; the velocities of these
    # quasi-static decks are ~1e-9 m/s, where float32 round-off is 1e-4 of them)
    for i in list(ref)[:: max(1, len(ref) // 10)]:
        with np.load(folder / npz_name(i, meta["nsteps"])) as f:
            for k in ("loc", "stress"):
                assert rel(f[k], ref[i][k]) <= 1e-4, (i, k)


def test_honor_scheme_and_cli(built, tmp_path, monkeypatch):
    deck = decks.load_deck("uniaxial_stress")
    deck["meta"] = dict(deck["meta"], scheme="usl")
    toml_decks.write_deck(deck, tmp_path)
    monkeypatch.chdir(tmp_path)
    assert D.MPM("deck.toml").solver.scheme == "usf"          # as the reference does
    assert D.MPM("deck.toml", honor_scheme=True).solver.scheme == "usl"
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ, PYTHONPATH=root + os.pathsep + os.environ.get("PYTHONPATH", ""))
    r = subprocess.run([sys.executable, "-m", "diffmpm_gb300", "-f", "deck.toml"], cwd=tmp_path,
                       env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    assert (tmp_path / "results" / deck["meta"]["title"] / npz_name(9, 10)).exists()


def test_async_output_equals_plain_reads(built):
    """Every output of solve_jit (copied behind the next steps, written by a
    host thread) equals a plain read after the same step."""
    got = {}
    solver, g, info = workloads.plain_scaleup(D, n=64, sim_steps=120)
    solver.out_steps = 7
    solver.writer_func = lambda a, t, **kw: got.__setitem__(a[1], a[0])
    final = solver.solve_jit(g)
    assert sorted(got) == list(range(0, 120, 7))
    sim = solver.simulation(g, reinit=True)
    solver._upload(sim)
    sim.initialize()
    done = 0
    for i in sorted(got):
        sim.step(i + 1 - done)
        done = i + 1
        for k in ("loc", "velocity", "stress", "strain"):
            a = sim.read(k)
            assert np.array_equal(got[i][k].reshape(a.shape), a), (i, k)
    sim.step(120 - done)
    assert np.array_equal(final["loc"].reshape(-1, 2), sim.read("loc"))


def test_async_output_writer_error_propagates(built):
    solver, g, info = workloads.plain_small(D, sim_steps=30)
    solver.out_steps = 5

    def bad(args, transforms, **kw):
        if args[1] == 10:
            raise RuntimeError("disk full")

    solver.writer_func = bad
    with pytest.raises(RuntimeError, match="disk full"):
        solver.solve_jit(g)


def test_output_enqueue_rejects_pageable_memory(built):
    solver, g, info = workloads.plain_small(D, sim_steps=2)
    sim = solver.simulation(g, reinit=True)
    solver._upload(sim)
    sim.initialize()

    from diffmpm_gb300 import _lib

    class Pageable:                       # ordinary NumPy memory, not page-locked
        buf = np.zeros(1 << 20, np.uint8)
        nbytes = buf.nbytes
        ptr = _lib.ptr(buf)

    with pytest.raises(D.MpmError):
        sim.output_enqueue(("loc",), Pageable)
    sim.close()


def test_one_dimensional_deck_end_to_end(built, tmp_path, monkeypatch):
    """The reference's 1-D example deck form (examples/input_1d.toml: node_ids
    constraints, no entity sets, SimpleMaterial, one element) runs through
    MPM on the GPU and matches the oracle bit for bit."""
    (tmp_path / "p.json").write_text("[[[0.5]]]")
    (tmp_path / "d.toml").write_text(
        '[meta]\ntitle = "bar"\ntype = "MPMExplicit"\ndimension = 1\nscheme = "usf"\n'
        'dt = 0.01\nnsteps = 200\nvelocity_update = true\n'
        '[output]\nformat = "npz"\nfolder = "results/"\nstep_frequency = 50\n'
        '[mesh]\ntype = "generator"\nnelements = 1\nelement_length = 1.0\n'
        'particle_element_ids = [0]\nelement = "Linear1D"\n'
        '[[mesh.constraints]]\nnode_ids = [0]\ndir = 0\nvelocity = 0.0\n'
        '[[materials]]\nid = 0\ndensity = 1\npoisson_ratio = 1\nE = 100\ntype = "SimpleMaterial"\n'
        '[[particles]]\nfile = "p.json"\nmaterial_id = 0\ninit_velocity = 0.1\n'
        '[external_loading]\ngravity = 0\n')
    monkeypatch.chdir(tmp_path)
    got = D.MPM("d.toml").solve()
    assert sorted(p.name for p in (tmp_path / "results" / "bar").iterdir()) == \
        [npz_name(i, 200) for i in range(0, 200, 50)]
    mat = O.SimpleMaterial({"E": 100, "density": 1})
    el = O.Linear1D(1, 1, 1.0, [(np.array([0]), O.Constraint(0, 0.0))])
    ps = O.Particles(np.array([0.5]).reshape(1, 1, 1), mat, np.zeros(1, dtype=np.int32))
    ps.velocity[:] = 0.1
    mesh = O.Mesh1D({"particles": [ps], "elements": el, "particle_surface_traction": []})
    ref = O.MPMExplicit(mesh, 0.01, scheme="usf", velocity_update=True, sim_steps=200).solve_jit(
        np.array([0.0]))
    for k in ("loc", "velocity", "stress", "strain"):
        assert np.array_equal(np.asarray(got[k]).reshape(-1), np.asarray(ref[k]).reshape(-1)), k
