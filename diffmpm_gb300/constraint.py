"""Velocity constraint (the reference's diffmpm/constraint.py:4-44)."""
from __future__ import annotations


class Constraint:
    """Constrain direction ``dir`` of the listed nodes to ``velocity``: on the GPU
    the nodal velocity is set to it, the momentum to mass * velocity and the
    acceleration to 0, in list order (diffmpm/constraint.py:29-44)."""

    def __init__(self, dir: int, velocity: float):
        if dir not in (0, 1):
            raise ValueError(f"dir must be 0 or 1, found {dir}")
        self.dir = dir
        self.velocity = velocity
