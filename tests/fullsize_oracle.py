"""Oracle runs of the benchmark configurations at full size, for the parity
tests in ``test_gpu_fullsize_parity.py``.

Each job runs in a worker process (started with ``spawn``, so none of them
inherits a CUDA context) and writes the fields it computed to an ``.npz``
file, returning the file name; the GPU side of the test runs meanwhile.

* ``numpy_job`` steps the float32 NumPy oracle (``oracle.mpm_oracle``) and
  saves the particle fields -- and, when asked, the nodal mass, velocity and
  acceleration -- after each listed step count.
* ``torch_job`` runs the torch restatement (``oracle.mpm_torch``, float32 or
  float64; many times faster at a million particles) for the long runs, and
  saves positions, velocities and stresses after the last step.
* ``linear_loss_f64`` is a linear functional of the end state of the float64
  torch restatement, for central differences of the differentiation run.
"""
from __future__ import annotations

import numpy as np

PARTICLE_FIELDS = ("loc", "velocity", "stress", "strain", "density", "volumetric_strain_centroid")
NODAL_FIELDS = ("mass", "velocity", "acceleration")


def _build(api, kind, kw):
    from diffmpm_gb300 import workloads
    if kind == "batch_member":
        spec = workloads.batch_specs(**kw.pop("specs_kw", {}))[kw.pop("member")]
        return workloads.batch_member(api, spec, **kw)
    return getattr(workloads, kind)(api, **kw)


def numpy_job(kind, kw, checkpoints, out_path, nodal=False, dtype="float32"):
    from oracle import mpm_oracle as O
    solver, g, info = _build(O, kind, dict(kw, dtype=np.dtype(dtype).type))
    p = solver.mesh.particles[0]
    nodes = solver.mesh.elements.nodes
    out = {}
    done = 0
    for c in sorted(checkpoints):
        for i in range(done, c):
            solver.step(i, g, reinit=True)
        done = c
        for k in PARTICLE_FIELDS:
            v = getattr(p, k)
            out[f"{c}/{k}"] = np.array(v, copy=True).reshape(len(p), -1).squeeze()
        if nodal:
            for k in NODAL_FIELDS:
                out[f"{c}/node_{k}"] = np.array(getattr(nodes, k), copy=True).reshape(
                    -1, 1 if k == "mass" else 2).squeeze()
    np.savez(out_path, **out)
    return out_path


def torch_job(kind, kw, steps, out_path, dtype="float32", threads=8):
    import torch
    from oracle import mpm_oracle as O
    from oracle import mpm_torch as T
    torch.set_num_threads(threads)
    solver, g, info = _build(O, kind, dict(kw, dtype=np.float64))
    sim, st = T.from_solver(solver, g, dtype=getattr(torch, dtype))
    with torch.no_grad():
        st = sim.run(st, steps)
    np.savez(out_path, loc=st["x"].numpy(), velocity=st["v"].numpy(), stress=st["sig"].numpy())
    return out_path


def linear_loss_f64(args):
    """<W, x_end> + <U, v_end> of the float64 torch restatement of the
    differentiation run with Young's modulus field ``E`` (runs in a worker)."""
    E, W, U, steps, threads = args
    import torch
    from oracle import mpm_oracle as O
    from oracle import mpm_torch as T
    torch.set_num_threads(threads)
    from diffmpm_gb300 import workloads
    o, g, info = workloads.differentiation(O, dtype=np.float64, sim_steps=steps)
    tsim, st0 = T.from_solver(o, g)
    with torch.no_grad():
        end = tsim.run(dict(st0), steps, E=torch.tensor(E, dtype=torch.float64))
    return float((end["x"].numpy() * W).sum() + (end["v"].numpy() * U).sum())
