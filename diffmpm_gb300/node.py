"""Nodal state container (the reference's diffmpm/node.py:9-125).

Host-side mirror of the nodal arrays, in the reference's shapes.  The GPU holds
the live state during a solve; ``velocity`` is uploaded as the initial nodal
velocity (it persists on nodes without mass, diffmpm/element.py:193-197).
"""
from __future__ import annotations

import numpy as np


class Nodes:
    def __init__(self, nnodes: int, loc):
        loc = np.asarray(loc, dtype=np.float32)
        if loc.ndim != 3:
            raise ValueError(f"`loc` should be of size (nnodes, 1, ndim); found {loc.shape}")
        self.nnodes = nnodes
        self.loc = loc
        self.velocity = np.zeros_like(loc)
        self.acceleration = np.zeros_like(loc)
        self.mass = np.ones((loc.shape[0], 1, 1), dtype=np.float32)
        self.momentum = np.zeros_like(loc)
        self.f_int = np.zeros_like(loc)
        self.f_ext = np.zeros_like(loc)
        self.f_damp = np.zeros_like(loc)

    def __len__(self):
        return self.nnodes

    def __repr__(self):
        return f"Nodes(n={self.nnodes})"
