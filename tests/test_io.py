"""The TOML deck loader (diffmpm_gb300.io.Config, the reference's
diffmpm/io.py:16-170) on the three benchmark decks, written back out in the
reference's file layout from the golden fixtures.  No GPU: only the parse."""
import json
import os

import numpy as np
import pytest

import diffmpm_gb300 as D
from diffmpm_gb300.io import Config
import decks
import toml_decks

NAMES = ["uniaxial_stress", "uniaxial_nodal_forces", "uniaxial_particle_traction"]


def fn_key(f):
    if isinstance(f, D.Linear):
        return ("Linear", f.id, tuple(f.xvalues), tuple(f.fxvalues))
    return (type(f).__name__, f.id)


@pytest.mark.parametrize("name", NAMES)
def test_config_matches_deck(tmp_path, name):
    deck = decks.load_deck(name)
    path = toml_decks.write_deck(deck, tmp_path)
    cfg = Config(path)
    pc = cfg.parsed_config
    assert pc["meta"] == deck["meta"] and pc["output"] == deck["output"]
    mesh = cfg.parse()
    assert isinstance(mesh, D.Mesh2D)
    el = mesh.elements
    assert isinstance(el, D.Quadrilateral4Node)
    assert el.nelements == tuple(deck["mesh"]["nelements"])
    assert np.allclose(el.el_len, deck["mesh"]["element_length"])
    assert len(el.constraints) == len(deck["mesh"]["constraints"])
    for (ids, c), want in zip(el.constraints, deck["mesh"]["constraints"]):
        assert list(ids) == list(decks.node_set_ids(deck, want["nset_ids"]))
        assert (c.dir, c.velocity) == (want["dir"], want["velocity"])
    assert len(mesh.particles) == len(deck["particles"])
    for ps, want in zip(mesh.particles, deck["particles"]):
        loc = np.asarray(want["loc"], np.float32)
        assert np.array_equal(ps.loc, loc)
        assert np.array_equal(ps.velocity, np.broadcast_to(
            np.asarray(want["init_velocity"], np.float32), loc.shape))
        m = deck["materials"][want["material_id"]]
        assert type(ps.material).__name__ == m["type"]
        assert ps.material.properties["density"] == m["density"]
    ext = deck["external_loading"]
    assert np.array_equal(pc["external_loading"]["gravity"], np.asarray(ext["gravity"], float))
    cnf = el.concentrated_nodal_forces
    assert len(cnf) == len(ext.get("concentrated_nodal_forces", []))
    for f, want in zip(cnf, ext.get("concentrated_nodal_forces", [])):
        assert list(f.node_ids) == list(decks.node_set_ids(deck, want["nset_ids"]))
        assert (f.dir, f.force) == (want["dir"], want["force"])
    tr = mesh.particle_tractions
    assert len(tr) == len(ext.get("particle_surface_traction", []))
    for t, want in zip(tr, ext.get("particle_surface_traction", [])):
        assert list(t.pids) == list(decks.particle_set_ids(deck, want["pset"], want["pset_ids"]))
        assert (t.dir, t.traction, list(t.pset)) == (want["dir"], want["traction"], want["pset"])
    # the same objects as the deck builder the golden tests use
    ref_solver_fns = [fn_key(f) for f in pc.get("math_functions", [])]
    assert ref_solver_fns == [("Linear", i, tuple(f["xvalues"]), tuple(f["fxvalues"]))
                              for i, f in enumerate(deck.get("math_functions", []))]


def test_relative_names_resolve_next_to_the_deck(tmp_path, monkeypatch):
    deck = decks.load_deck("uniaxial_stress")
    path = toml_decks.write_deck(deck, tmp_path / "case")
    monkeypatch.chdir(tmp_path)          # the files are not in the working directory
    mesh = Config(path).parse()
    assert len(mesh.particles[0].loc) == len(deck["particles"][0]["loc"])


def test_one_dimensional_example_form(tmp_path):
    """The reference's 1-D example deck form: node_ids constraints, no entity
    sets, scalar nelements / element_length / gravity / init_velocity."""
    (tmp_path / "p.json").write_text(json.dumps([[[0.5]]]))
    (tmp_path / "d.toml").write_text(
        '[meta]\ntitle = "bar"\ntype = "MPMExplicit"\ndimension = 1\nscheme = "usl"\n'
        'dt = 0.01\nnsteps = 10\nvelocity_update = true\n'
        '[output]\nformat = "none"\nfolder = "results/"\nstep_frequency = 1\n'
        '[mesh]\ntype = "generator"\nnelements = 1\nelement_length = 1.0\n'
        'particle_element_ids = [0]\nelement = "Linear1D"\n'
        '[[mesh.constraints]]\nnode_ids = [0]\ndir = 0\nvelocity = 0.0\n'
        '[[materials]]\nid = 0\ndensity = 1\npoisson_ratio = 1\nE = 100\ntype = "SimpleMaterial"\n'
        '[[particles]]\nfile = "p.json"\nmaterial_id = 0\ninit_velocity = 0.1\n'
        '[external_loading]\ngravity = 0\n')
    mesh = Config(tmp_path / "d.toml").parse()
    assert isinstance(mesh, D.Mesh1D) and isinstance(mesh.elements, D.Linear1D)
    assert mesh.elements.nelements == 1 and list(mesh.elements.constraints[0][0]) == [0]
    assert mesh.particles[0].velocity.reshape(-1).tolist() == [pytest.approx(0.1)]


def _edit(tmp_path, old, new, name="uniaxial_particle_traction"):
    path = toml_decks.write_deck(decks.load_deck(name), tmp_path)
    text = path.read_text()
    assert old in text
    path.write_text(text.replace(old, new))
    return path


def test_unsupported_function_type(tmp_path):
    path = _edit(tmp_path, 'type = "Linear"', 'type = "Sine"')
    with pytest.raises(NotImplementedError):
        Config(path)


def test_unsupported_mesh_type(tmp_path):
    path = _edit(tmp_path, 'type = "generator"', 'type = "file"')
    with pytest.raises(NotImplementedError):
        Config(path)


def test_unknown_material_raises(tmp_path):
    path = _edit(tmp_path, 'type = "LinearElastic"', 'type = "Plastic"')
    with pytest.raises(AttributeError):
        Config(path)


def test_mpm_rejects_bad_output_and_solver(tmp_path):
    path = _edit(tmp_path, 'format = "npz"', 'format = "vtk"')
    with pytest.raises(ValueError, match="output format"):
        D.MPM(path)
    path = _edit(tmp_path / "b", 'type = "MPMExplicit"', 'type = "MPMImplicit"')
    with pytest.raises(ValueError, match="solver"):
        D.MPM(path)


def test_npz_writer_file_names(tmp_path):
    """particles_<step>.npz with the step zero-padded to the digits of
    max_steps (the names the reference's benchmark readers open)."""
    import numpy as np
    from diffmpm_gb300.writers import NPZWriter
    w = NPZWriter()
    a = {"loc": np.zeros((2, 2), np.float32)}
    for step, max_steps, name in [(0, 1000, "particles_0000.npz"), (5, 1000, "particles_0005.npz"),
                                  (10, 1000, "particles_0010.npz"), (999, 1000, "particles_0999.npz"),
                                  (0, 10, "particles_00.npz"), (7, 999, "particles_007.npz"),
                                  (12345, 100, "particles_12345.npz")]:
        w.write((a, step), None, out_dir=tmp_path / str(max_steps), max_steps=max_steps)
        f = tmp_path / str(max_steps) / name
        assert f.exists(), name
        np.testing.assert_array_equal(np.load(f)["loc"], a["loc"])
