"""Input decks: the reference's TOML configuration (diffmpm/io.py:16-170).

``Config(path).parse()`` reads the TOML deck, the entity-set JSON and the
particle JSON files it names, and builds this package's Mesh / Particles /
element / material / force objects, which the GPU solver consumes.  The
parsed pieces land in ``parsed_config`` under the reference's keys ("meta",
"output", "materials", "particles", "math_functions", "external_loading",
"particle_surface_traction", "elements").

File names in the deck are opened as given (relative to the working
directory, as the reference does, diffmpm/io.py:25,67); a name that does not
exist there is looked up next to the deck.  Two forms of the reference's own
1-D example deck (examples/input_1d.toml) are accepted as well: constraints
that list ``node_ids`` instead of ``nset_ids``, and a deck without
``mesh.entity_sets`` when no set is referenced.
"""
from __future__ import annotations

import json
import tomllib
from pathlib import Path

import numpy as np

from . import element as _element
from . import material as _material
from . import mesh as _mesh
from .constraint import Constraint
from .forces import NodalForce, ParticleTraction
from .functions import Linear, Unit
from .particle import Particles

__all__ = ["Config"]


class Config:
    """Parser of one TOML deck (diffmpm/io.py:16-36)."""

    def __init__(self, filepath):
        self._filepath = Path(filepath)
        self.parsed_config = {}
        self.parse()

    def _path(self, name) -> Path:
        p = Path(name)
        if p.exists() or p.is_absolute():
            return p
        q = self._filepath.parent / p
        return q if q.exists() else p

    def parse(self):
        """Read the deck and return the mesh (diffmpm/io.py:21-36)."""
        with open(self._filepath, "rb") as f:
            self._fileconfig = tomllib.load(f)
        cfg = self._fileconfig
        es = cfg["mesh"].get("entity_sets")
        self.entity_sets = (json.loads(self._path(es).read_text()) if es is not None
                            else {"node_sets": {}, "particle_sets": []})
        self.parsed_config["meta"] = cfg["meta"]
        self.parsed_config["output"] = cfg["output"]
        self._parse_materials(cfg)
        self._parse_particles(cfg)
        if "math_functions" in cfg:
            self._parse_math_functions(cfg)
        self._parse_external_loading(cfg)
        return self._parse_mesh(cfg)

    # entity sets (diffmpm/io.py:38-52)
    def _get_node_set_ids(self, set_ids):
        ids = []
        for s in set_ids:
            ids.extend(self.entity_sets["node_sets"][str(s)])
        return np.asarray(ids, dtype=np.int64)

    def _get_particle_set_ids(self, set_type, set_nos, set_ids):
        ids = []
        for n in set_nos:
            for s in set_ids:
                ids.extend(self.entity_sets["particle_sets"][n][str(s)])
        return np.asarray(ids, dtype=np.int64)

    def _parse_materials(self, cfg):
        """One material object per [[materials]] table, class named by its
        ``type`` (diffmpm/io.py:60-67)."""
        mats = []
        for m in cfg["materials"]:
            props = {k: v for k, v in m.items() if k != "type"}
            mats.append(getattr(_material, m["type"])(props))
        self.parsed_config["materials"] = mats

    def _parse_particles(self, cfg):
        """Particle locations from JSON, zero element ids, the deck's initial
        velocity broadcast to every particle (diffmpm/io.py:69-79)."""
        sets = []
        for p in cfg["particles"]:
            loc = np.asarray(json.loads(self._path(p["file"]).read_text()), dtype=np.float64)
            ps = Particles(loc, self.parsed_config["materials"][p["material_id"]],
                           np.zeros(loc.shape[0], dtype=np.int32))
            ps.velocity[:] = np.asarray(p["init_velocity"], dtype=np.float64)
            sets.append(ps)
        self.parsed_config["particles"] = sets

    def _parse_math_functions(self, cfg):
        """Linear functions only; other types raise NotImplementedError
        (diffmpm/io.py:81-95)."""
        fns = []
        for i, f in enumerate(cfg["math_functions"]):
            if f["type"] != "Linear":
                raise NotImplementedError("Function type other than `Linear` not yet supported")
            fns.append(Linear(i, np.asarray(f["xvalues"]), np.asarray(f["fxvalues"])))
        self.parsed_config["math_functions"] = fns

    def _function(self, c):
        if "math_function_id" in c:
            return self.parsed_config["math_functions"][c["math_function_id"]]
        return Unit(-1)

    def _parse_external_loading(self, cfg):
        """Gravity, concentrated nodal forces and particle surface tractions
        (diffmpm/io.py:97-144)."""
        el = cfg["external_loading"]
        loading = {"gravity": np.asarray(el["gravity"], dtype=np.float64),
                   "concentrated_nodal_forces": []}
        for c in el.get("concentrated_nodal_forces", []):
            loading["concentrated_nodal_forces"].append(NodalForce(
                node_ids=self._get_node_set_ids(c["nset_ids"]), function=self._function(c),
                dir=c["dir"], force=c["force"]))
        tractions = []
        for t in el.get("particle_surface_traction", []):
            tractions.append(ParticleTraction(
                pset=t["pset"], pids=self._get_particle_set_ids("particle", t["pset"], t["pset_ids"]),
                function=self._function(t), dir=t["dir"], traction=t["traction"]))
        self.parsed_config["external_loading"] = loading
        self.parsed_config["particle_surface_traction"] = tractions

    def _parse_mesh(self, cfg):
        """Generated meshes only (diffmpm/io.py:146-170)."""
        m = cfg["mesh"]
        el_cls = getattr(_element, m["element"])
        mesh_cls = getattr(_mesh, f"Mesh{cfg['meta']['dimension']}D")
        cons = []
        for c in m.get("constraints", []):
            ids = (self._get_node_set_ids(c["nset_ids"]) if "nset_ids" in c
                   else np.asarray(c["node_ids"], dtype=np.int64))
            cons.append((ids, Constraint(c["dir"], c["velocity"])))
        if m["type"] != "generator":
            raise NotImplementedError("Mesh type other than `generator` not yet supported.")
        nel = m["nelements"]
        elements = el_cls(nel, int(np.prod(np.asarray(nel))), m["element_length"], cons,
                          concentrated_nodal_forces=self.parsed_config["external_loading"][
                              "concentrated_nodal_forces"])
        self.parsed_config["elements"] = elements
        return mesh_cls(self.parsed_config)
