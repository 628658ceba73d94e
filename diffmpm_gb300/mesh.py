"""Mesh containers (the reference's diffmpm/mesh.py:13-126).

The reference applies every element/particle method once per particle set
(mesh.py:31-58), which with several sets resets the nodal sums per set.  This
build advances all sets as one population with per-particle material ids, so
every set contributes to the nodal sums.
"""
from __future__ import annotations


class _MeshBase:
    ndim = 2

    def __init__(self, config: dict):
        self.particles = list(config["particles"])
        self.elements = config["elements"]
        self.particle_tractions = list(config.get("particle_surface_traction", []))
        self.particle_velocity_constraints = list(config.get("particle_velocity_constraints", []))


class Mesh1D(_MeshBase):
    ndim = 1


class Mesh2D(_MeshBase):
    ndim = 2
