"""PyTorch autograd over the GPU step: forward = checkpointed run, backward =
the hand-written adjoint (include/diffmpm_gb300.h: mpm_record, mpm_adjoint).

The reference differentiates ``solve_jit`` with ``jax.grad``
(examples/optim_1d.py:33-41,55).  Here

    x_end, v_end = explicit_run(mpm, gravity, E)

runs ``mpm.sim_steps`` steps from the initial state held by ``mpm`` (an
``MPMExplicit``) with the per-particle Young's modulus ``E`` (a torch tensor,
CPU or CUDA, original particle order) and returns the final positions and
velocities; ``torch.autograd.grad`` / ``.backward()`` through them calls the
adjoint.  Gradients flow to ``E`` and, when given, to the initial positions
``loc`` and velocities ``velocity``.  Arithmetic is float32, as the forward.

Every forward records into a simulation of its own, leased from ``mpm``'s
pool (``MPMExplicit.lease_simulation``) and returned to it when the autograd
graph that holds the forward is freed, so forwards and backwards may
interleave freely: two forwards before their backwards, two losses on one
graph, or a forward-only evaluation inside a training step.  A loop that runs
forward then backward cycles through a pool of two simulations (the previous
iteration's graph is freed only once the next forward has returned), keeping
their allocations and captured step graphs.
"""
from __future__ import annotations

import numpy as np
import torch


def _dev_f32(t, device):
    return t.detach().to(device=device, dtype=torch.float32).contiguous()


class ExplicitRun(torch.autograd.Function):
    @staticmethod
    def forward(ctx, E, loc, velocity, mpm, gravity, nsteps, checkpoint_steps):
        lease = mpm.lease_simulation(gravity, reinit=True)
        sim = lease.sim
        mpm._upload(sim)
        dev = E.device if E.is_cuda else None
        put = (lambda t: _dev_f32(t, dev)) if dev is not None else (
            lambda t: t.detach().cpu().numpy().astype(np.float32))
        d = sim.ndim
        sim.write("youngs_modulus", put(E))
        if loc is not None:
            sim.write("loc", put(loc.reshape(-1, d)))
        if velocity is not None:
            sim.write("velocity", put(velocity.reshape(-1, d)))
        sim.initialize()
        sim.record(nsteps, checkpoint_steps)
        n = sim.n
        if dev is not None:
            x = torch.empty((n, d), dtype=torch.float32, device=dev)
            v = torch.empty((n, d), dtype=torch.float32, device=dev)
            sim.read("loc", out=x)
            sim.read("velocity", out=v)
        else:
            x = torch.from_numpy(sim.read("loc"))
            v = torch.from_numpy(sim.read("velocity"))
        ctx.lease = lease
        ctx.sim = sim
        ctx.dev = dev
        ctx.want = ("youngs_modulus",) + (("loc",) if loc is not None else ()) + (
            ("velocity",) if velocity is not None else ())
        ctx.shapes = (E.shape, None if loc is None else loc.shape,
                      None if velocity is None else velocity.shape)
        ctx.dtypes = (E.dtype, None if loc is None else loc.dtype,
                      None if velocity is None else velocity.dtype)
        return x, v

    @staticmethod
    def backward(ctx, gx, gv):
        dev = ctx.dev
        shape = (ctx.sim.n, ctx.sim.ndim)
        if dev is not None:
            seed_x = (torch.zeros(shape, dtype=torch.float32, device=dev) if gx is None
                      else _dev_f32(gx, dev))
            seed_v = None if gv is None else _dev_f32(gv, dev)
        else:
            seed_x = (np.zeros(shape, np.float32) if gx is None
                      else gx.detach().cpu().numpy().astype(np.float32))
            seed_v = None if gv is None else gv.detach().cpu().numpy().astype(np.float32)
        out = ctx.sim.adjoint(seed_x, seed_v, want=ctx.want)
        grads = []
        for key, shape, dtype in zip(("youngs_modulus", "loc", "velocity"), ctx.shapes, ctx.dtypes):
            if key not in out:
                grads.append(None)
                continue
            g = out[key] if dev is not None else torch.from_numpy(out[key])
            grads.append(g.reshape(shape).to(dtype))
        return grads[0], grads[1], grads[2], None, None, None, None


def explicit_run(mpm, gravity, E, loc=None, velocity=None, nsteps=None, checkpoint_steps=100):
    """Final (positions, velocities) of ``nsteps`` (default ``mpm.sim_steps``)
    steps, differentiable w.r.t. ``E`` and the optional ``loc``/``velocity``."""
    g = torch.as_tensor(np.asarray(gravity, dtype=np.float64))
    return ExplicitRun.apply(E, loc, velocity, mpm, tuple(g.tolist()),
                             int(mpm.sim_steps if nsteps is None else nsteps), int(checkpoint_steps))
