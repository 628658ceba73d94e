"""Output writers (the reference's diffmpm/writers.py:14-54)."""
from __future__ import annotations

import logging
from pathlib import Path

import numpy as np

logger = logging.getLogger(__name__)

__all__ = ["EmptyWriter", "NPZWriter"]


class EmptyWriter:
    """Writes nothing (diffmpm/writers.py:22-28)."""

    def write(self, args, transforms=None, **kwargs):
        pass


class NPZWriter:
    """Writes ``particles_<step>.npz`` with the step zero-padded to
    ``int(log10(max_steps)) + 1`` digits (diffmpm/writers.py:30-54)."""

    def write(self, args, transforms=None, **kwargs):
        arrays, step = args
        max_digits = int(np.log10(kwargs["max_steps"])) + 1
        req_zeros = max_digits - 1 if step == 0 else max_digits - (int(np.log10(step)) + 1)
        fileno = f"{'0' * req_zeros}{step}"
        filepath = Path(kwargs["out_dir"]).joinpath(f"particles_{fileno}.npz")
        filepath.parent.mkdir(parents=True, exist_ok=True)
        np.savez(filepath, **arrays)
        logger.info(f"Saved particle data for step {step} at {filepath}")
