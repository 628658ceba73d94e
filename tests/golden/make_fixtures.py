"""Generate the golden fixtures under tests/golden/ from the reference checkout.

Run once where the reference is mounted:

    python tests/golden/make_fixtures.py <reference checkout>

For each end-to-end benchmark in ``benchmarks/2d/<name>/`` of diffmpm it reads
the TOML input deck, the entity-set JSON and the particle JSON, and the golden
assertions of ``test_benchmark.py`` (read as text: the npz file name, the stress
component, min/max and the expected value with its rounding decimals).  It writes
``tests/golden/<name>.json`` holding the parsed deck and the goldens.  The
reference's unit-test known answers are restated by hand in
``tests/test_oracle_kat.py`` with file:line citations, so they need no fixture.
"""
from __future__ import annotations

import json
import re
import sys
import tomllib
from pathlib import Path

BENCHMARKS = ("uniaxial_stress", "uniaxial_nodal_forces", "uniaxial_particle_traction")

# jnp.round(result["stress"][0, :, 0].min() - 0.5925210678182377, 6) == 0.0
_ASSERT = re.compile(
    r'result\["stress"\]\[0,\s*:,\s*(\d)\]\.(min|max)\(\)\s*-\s*([-+0-9.eE]+)\s*\)?\s*,\s*(\d+)'
)
_LOAD = re.compile(r'jnp\.load\("results/([^"]+)/particles_(\d+)\.npz"\)')
_TRUE = re.compile(r"true_stress_(xx|yy)\s*=\s*([-+0-9.eE]+)")
_TRUE_ASSERT = re.compile(
    r'result\["stress"\]\[0,\s*:,\s*(\d)\]\.(min|max)\(\)\s*-\s*true_stress_(xx|yy)\s*,\s*(\d+)'
)


def parse_goldens(text: str):
    goldens = []
    current = None
    trues = dict(_TRUE.findall(text))
    for line in text.splitlines():
        m = _LOAD.search(line)
        if m:
            current = int(m.group(2))
            continue
        m = _ASSERT.search(line)
        if m and current is not None:
            comp, op, val, dp = m.groups()
            goldens.append({"file_index": current, "component": int(comp), "op": op,
                            "value": float(val), "decimals": int(dp)})
            continue
        m = _TRUE_ASSERT.search(line)
        if m and current is not None:
            comp, op, name, dp = m.groups()
            goldens.append({"file_index": current, "component": int(comp), "op": op,
                            "value": float(trues[name]), "decimals": int(dp)})
    return goldens


def build(ref: Path, name: str) -> dict:
    d = ref / "benchmarks" / "2d" / name
    toml_path = next(d.glob("*.toml"))
    with open(toml_path, "rb") as f:
        cfg = tomllib.load(f)
    entity_sets = json.loads((d / cfg["mesh"]["entity_sets"]).read_text())
    particles = []
    for p in cfg["particles"]:
        loc = json.loads((d / p["file"]).read_text())
        particles.append({"loc": loc, "material_id": p["material_id"],
                          "init_velocity": p["init_velocity"]})
    return {
        "name": name,
        "source": f"benchmarks/2d/{name}/{toml_path.name}",
        "meta": cfg["meta"],
        "output": cfg["output"],
        "mesh": {k: v for k, v in cfg["mesh"].items() if k != "entity_sets"},
        "entity_sets": entity_sets,
        "materials": cfg["materials"],
        "particles": particles,
        "external_loading": cfg["external_loading"],
        "math_functions": cfg.get("math_functions", []),
        "goldens": parse_goldens((d / "test_benchmark.py").read_text()),
    }


def main(argv):
    if len(argv) != 2:
        raise SystemExit(f"usage: {argv[0]} <path of the diffmpm reference checkout>")
    ref = Path(argv[1])
    out = Path(__file__).resolve().parent
    for name in BENCHMARKS:
        fx = build(ref, name)
        assert fx["goldens"], f"no goldens parsed for {name}"
        (out / f"{name}.json").write_text(json.dumps(fx, indent=1) + "\n")
        print(f"{name}: {len(fx['particles'][0]['loc'])} particles, "
              f"{len(fx['goldens'])} golden assertions")


if __name__ == "__main__":
    main(sys.argv)
