"""Build a simulation from a parsed input deck (tests/golden/*.json).

The deck layout is the reference's TOML input (diffmpm/io.py:16-170).  ``api``
is any module exposing the reference's class names -- the oracle
(``oracle.mpm_oracle``) or the product (``diffmpm_gb300``) -- so the same deck
drives both.  As in the reference's ``MPM`` wrapper (diffmpm/__init__.py:30-38)
the deck's ``meta.scheme`` is ignored unless ``honor_scheme`` is set.
"""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden"


def load_deck(name: str) -> dict:
    return json.loads((GOLDEN / f"{name}.json").read_text())


def node_set_ids(deck, set_ids):
    out = []
    for s in set_ids:
        out.extend(deck["entity_sets"]["node_sets"][str(s)])
    return np.asarray(out, dtype=np.int64)


def particle_set_ids(deck, set_nos, set_ids):
    out = []
    for n in set_nos:
        for s in set_ids:
            out.extend(deck["entity_sets"]["particle_sets"][n][str(s)])
    return np.asarray(out, dtype=np.int64)


def build(api, deck, writer_func=None, honor_scheme=False, sim_steps=None, **kw):
    """Return ``(solver, gravity)`` for ``deck`` built with ``api``'s classes."""
    fns = []
    for i, f in enumerate(deck.get("math_functions", [])):
        assert f["type"] == "Linear"
        fns.append(api.Linear(i, np.asarray(f["xvalues"]), np.asarray(f["fxvalues"])))
    mats = []
    for m in deck["materials"]:
        props = {k: v for k, v in m.items() if k != "type"}
        mats.append(getattr(api, m["type"])(props))
    psets = []
    for p in deck["particles"]:
        loc = np.asarray(p["loc"], dtype=np.float64)
        ps = api.Particles(loc, mats[p["material_id"]], np.zeros(loc.shape[0], dtype=np.int32), **kw)
        ps.velocity[:] = np.asarray(p["init_velocity"], dtype=np.float64)
        psets.append(ps)
    el = deck["external_loading"]
    cnfs = []
    for c in el.get("concentrated_nodal_forces", []):
        fn = fns[c["math_function_id"]] if "math_function_id" in c else api.Unit(-1)
        cnfs.append(api.NodalForce(node_ids=node_set_ids(deck, c["nset_ids"]), function=fn,
                                   dir=c["dir"], force=c["force"]))
    tractions = []
    for t in el.get("particle_surface_traction", []):
        fn = fns[t["math_function_id"]] if "math_function_id" in t else api.Unit(-1)
        tractions.append(api.ParticleTraction(
            pset=t["pset"], pids=particle_set_ids(deck, t["pset"], t["pset_ids"]),
            function=fn, dir=t["dir"], traction=t["traction"]))
    mesh_cfg = deck["mesh"]
    cons = [(node_set_ids(deck, c["nset_ids"]), api.Constraint(c["dir"], c["velocity"]))
            for c in mesh_cfg["constraints"]]
    nel = mesh_cfg["nelements"]
    el_cls = getattr(api, mesh_cfg["element"])
    elements = el_cls(nel, int(np.prod(nel)), mesh_cfg["element_length"], cons,
                      concentrated_nodal_forces=cnfs, **kw)
    mesh_cls = getattr(api, f"Mesh{deck['meta']['dimension']}D")
    mesh = mesh_cls({"particles": psets, "elements": elements,
                     "particle_surface_traction": tractions})
    meta = deck["meta"]
    extra = {"scheme": meta.get("scheme", "usf")} if honor_scheme else {}
    solver = api.MPMExplicit(
        mesh, meta["dt"], velocity_update=meta["velocity_update"],
        sim_steps=sim_steps if sim_steps is not None else meta["nsteps"],
        out_steps=deck["output"]["step_frequency"], writer_func=writer_func, **extra)
    return solver, np.asarray(el["gravity"], dtype=np.float64)


def check_goldens(deck, stress_at):
    """Assert every golden of ``deck``; ``stress_at[file_index]`` is the
    (nsets, Np, 6) stress array the reference writes to that npz file."""
    for g in deck["goldens"]:
        s = np.asarray(stress_at[g["file_index"]], dtype=np.float32)[0, :, g["component"]]
        got = getattr(s, g["op"])()
        # the reference subtracts in float32 and rounds with jnp.round
        diff = np.float32(got) - np.float32(g["value"])
        assert np.round(diff, g["decimals"]) == 0.0, (g, float(got))
