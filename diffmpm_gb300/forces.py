"""External-force descriptors (the reference's diffmpm/forces.py:9-61)."""
from __future__ import annotations

from typing import NamedTuple


class NodalForce(NamedTuple):
    """Concentrated nodal force f(t) * force on ``node_ids`` in ``dir``
    (diffmpm/forces.py:9-18, applied as in element.py:270-284)."""

    node_ids: object
    function: object
    dir: int
    force: float


class ParticleTraction(NamedTuple):
    """Traction on particles ``pids`` of the particle sets ``pset``
    (diffmpm/forces.py:26-41, applied as in mesh.py:60-77)."""

    pset: object
    pids: object
    function: object
    dir: int
    traction: float
