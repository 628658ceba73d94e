"""Write a parsed input deck (tests/golden/<name>.json) back out as the
reference's file layout: a TOML deck, ``entity_sets.json`` and one particle
JSON per set (the layout of benchmarks/2d/<name>/ in diffmpm), so the TOML
loader can be run on it."""
from __future__ import annotations

import json
from pathlib import Path


def _value(v):
    if isinstance(v, bool):
        return "true" if v else "false"
    if isinstance(v, (int, float)):
        return repr(v)
    if isinstance(v, str):
        return json.dumps(v)
    if isinstance(v, (list, tuple)):
        return "[" + ", ".join(_value(x) for x in v) + "]"
    raise TypeError(type(v))


def _table(lines, header, d):
    lines.append(header)
    for k, v in d.items():
        if not isinstance(v, dict) and not (isinstance(v, list) and v and isinstance(v[0], dict)):
            lines.append(f"{k} = {_value(v)}")
    lines.append("")


def write_deck(deck: dict, folder: Path, name: str = "deck.toml") -> Path:
    folder = Path(folder)
    folder.mkdir(parents=True, exist_ok=True)
    (folder / "entity_sets.json").write_text(json.dumps(deck["entity_sets"]))
    lines = []
    _table(lines, "[meta]", deck["meta"])
    _table(lines, "[output]", deck["output"])
    _table(lines, "[mesh]", dict(deck["mesh"], entity_sets="entity_sets.json"))
    for c in deck["mesh"].get("constraints", []):
        _table(lines, "[[mesh.constraints]]", c)
    for m in deck["materials"]:
        _table(lines, "[[materials]]", m)
    for i, p in enumerate(deck["particles"]):
        fname = f"particles-{i}.json"
        (folder / fname).write_text(json.dumps(p["loc"]))
        _table(lines, "[[particles]]", {"file": fname, "material_id": p["material_id"],
                                         "init_velocity": p["init_velocity"]})
    el = deck["external_loading"]
    _table(lines, "[external_loading]", el)
    for key in ("concentrated_nodal_forces", "particle_surface_traction"):
        for c in el.get(key, []):
            _table(lines, f"[[external_loading.{key}]]", c)
    for f in deck.get("math_functions", []):
        _table(lines, "[[math_functions]]", f)
    path = folder / name
    path.write_text("\n".join(lines))
    return path
