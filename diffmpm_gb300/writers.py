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


class AsyncOutput:
    """Writes outputs on a host thread while the GPU keeps stepping.

    ``submit(i)`` enqueues the copy of ``fields`` at the current step into one
    of ``nbuf`` pinned host buffers (mpm_output_enqueue) and hands the buffer
    to a writer thread, which waits for the copy, assembles the reference's
    output dict with ``assemble`` and calls
    ``writer_func((arrays, i), None, out_dir=..., max_steps=...)`` -- the call
    the reference's host callback makes (diffmpm/solver.py:187-210).  The
    writer receives arrays of its own (copied out of the pinned buffer), so it
    may keep them.  Files are written in step order; an exception raised by
    the writer is raised again by the next ``submit`` or by ``close``.
    """

    def __init__(self, sim, fields, assemble, writer_func, nbuf=3, **writer_kwargs):
        from concurrent.futures import ThreadPoolExecutor

        from .engine import PinnedBuffer
        self.sim, self.fields = sim, tuple(fields)
        self.assemble, self.writer_func, self.kwargs = assemble, writer_func, writer_kwargs
        nbytes = sum(4 * sim.n * sim.ncomp(f) for f in self.fields)
        self.buffers = [PinnedBuffer(nbytes) for _ in range(nbuf)]
        self.pending = [None] * nbuf
        self.count = 0
        self.pool = ThreadPoolExecutor(max_workers=1, thread_name_prefix="mpm-output")

    def submit(self, step):
        k = self.count % len(self.buffers)
        if self.pending[k] is not None:
            self.pending[k].result()          # the buffer's previous file is written
        ticket = self.sim.output_enqueue(self.fields, self.buffers[k])
        self.pending[k] = self.pool.submit(self._write, k, ticket, step)
        self.count += 1

    def _write(self, k, ticket, step):
        self.sim.output_wait(ticket)
        views = self.sim.output_views(self.fields, self.buffers[k])
        arrays = self.assemble({f: v.copy() for f, v in views.items()})
        self.writer_func((arrays, step), None, **self.kwargs)

    def close(self):
        try:
            for f in self.pending:
                if f is not None:
                    f.result()
        finally:
            self.pool.shutdown(wait=True)
            for b in self.buffers:
                b.close()
            self.buffers = []
