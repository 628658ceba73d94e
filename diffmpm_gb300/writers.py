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
    """Writes ``particles_<step>.npz`` into ``out_dir``, the step number
    zero-padded to as many digits as ``max_steps`` has (the file names of
    diffmpm/writers.py:30-54, which the reference's benchmark readers open)."""

    def write(self, args, transforms=None, **kwargs):
        arrays, step = args
        width = len(str(int(kwargs["max_steps"])))
        target = Path(kwargs["out_dir"]) / f"particles_{int(step):0{width}d}.npz"
        target.parent.mkdir(parents=True, exist_ok=True)
        np.savez(target, **arrays)
        logger.info("step %d written to %s", step, target)


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
