"""Time functions (the reference's diffmpm/functions.py:7-49).

The values are evaluated on the GPU each step; these classes only describe them.
"""
from __future__ import annotations

import numpy as np


class Function:
    def __init__(self, id):
        self.id = id


class Unit(Function):
    """f(t) = 1 (diffmpm/functions.py:16-31)."""


class Linear(Function):
    """Piecewise-linear f(t), held constant outside the table
    (diffmpm/functions.py:33-49, ``jnp.interp``)."""

    def __init__(self, id, xvalues, fxvalues):
        self.xvalues = np.asarray(xvalues, dtype=np.float64).reshape(-1)
        self.fxvalues = np.asarray(fxvalues, dtype=np.float64).reshape(-1)
        if self.xvalues.shape != self.fxvalues.shape or self.xvalues.size == 0:
            raise ValueError("xvalues and fxvalues must be non-empty and of equal length")
        super().__init__(id)
