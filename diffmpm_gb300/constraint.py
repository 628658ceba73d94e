"""Velocity constraint (the reference's diffmpm/constraint.py:4-44)."""
from __future__ import annotations

from typing import NamedTuple


class Constraint:
    """Constrain direction ``dir`` of the listed nodes to ``velocity``: on the GPU
    the nodal velocity is set to it, the momentum to mass * velocity and the
    acceleration to 0, in list order (diffmpm/constraint.py:29-44)."""

    def __init__(self, dir: int, velocity: float):
        if dir not in (0, 1):
            raise ValueError(f"dir must be 0 or 1, found {dir}")
        self.dir = dir
        self.velocity = velocity


class ParticleVelocityConstraint(NamedTuple):
    """Velocity ``velocity`` in direction ``dir`` of particles ``pids`` of the
    particle sets ``pset``, imposed on the GPU after every particle velocity
    update.  An extension: the reference leaves particle velocity constraints
    as a TODO (diffmpm/scheme.py:67); the list goes into the mesh config under
    "particle_velocity_constraints", next to "particle_surface_traction"."""

    pset: object
    pids: object
    dir: int
    velocity: float
