"""``MPM``: a simulation from a TOML deck (the reference's diffmpm/__init__.py:13-47).

    MPM("mpm-uniaxial-stress.toml").solve()

builds the mesh with :class:`diffmpm_gb300.io.Config`, an :class:`MPMExplicit`
with the deck's dt, velocity_update, nsteps and output frequency, writes
``particles_<step>.npz`` into ``<output.folder>/<meta.title>`` when
``output.format`` is "npz", and runs ``solve_jit`` with the deck's gravity.

The reference never passes ``meta.scheme`` on, so every deck runs USF
(diffmpm/__init__.py:30-38).  This class does the same unless
``honor_scheme=True``.
"""
from __future__ import annotations

from pathlib import Path

from . import writers
from .io import Config
from .solver import MPMExplicit

__all__ = ["MPM"]


class MPM:
    def __init__(self, filepath, honor_scheme: bool = False):
        self._config = Config(filepath)
        mesh = self._config.parse()
        pc = self._config.parsed_config
        out_dir = Path(pc["output"]["folder"]).joinpath(pc["meta"]["title"])
        fmt = pc["output"].get("format", None)
        if fmt is None or fmt.lower() == "none":
            writer_func = None
        elif fmt == "npz":
            writer_func = writers.NPZWriter().write
        else:
            raise ValueError(f"Specified output format not supported: {fmt}")
        if pc["meta"]["type"] != "MPMExplicit":
            raise ValueError("Wrong type of solver specified.")
        extra = {"scheme": pc["meta"].get("scheme", "usf")} if honor_scheme else {}
        self.solver = MPMExplicit(
            mesh, pc["meta"]["dt"], velocity_update=pc["meta"]["velocity_update"],
            sim_steps=pc["meta"]["nsteps"], out_steps=pc["output"]["step_frequency"],
            out_dir=out_dir, writer_func=writer_func, **extra)

    def solve(self):
        """Run the deck with solve_jit semantics (diffmpm/__init__.py:42-47)."""
        return self.solver.solve_jit(self._config.parsed_config["external_loading"]["gravity"])
