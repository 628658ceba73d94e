"""Error of the float32 CUDA step against a float64 run of the oracle, for
each benchmark configuration (reduced where the float64 oracle would take
minutes).

For every field the normwise relative error of the GPU against float64 is
set beside that of the float32 oracle (the reference's own float32 program)
against float64; the GPU must be within 3x of the latter or below 1e-5.  A
field that is exactly zero in float64 (the stress of a block in free fall,
whose strain rates float64 flushes and float32 does not) is reported as the
RMS absolute difference instead, marked "abs".  The table is printed at the
end of the pytest run.
"""
import numpy as np
import pytest

import diffmpm_gb300 as D
from diffmpm_gb300 import workloads
from oracle import mpm_oracle as O

pytestmark = pytest.mark.gpu

FLOOR = 1e-5
TABLE = []


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def fields_of(p):
    return {"loc": p.loc.reshape(-1, 2), "velocity": p.velocity.reshape(-1, 2),
            "stress": p.stress.reshape(-1, 6)[:, [0, 1, 3]]}


def gpu_fields(sim):
    return {"loc": sim.read("loc"), "velocity": sim.read("velocity"),
            "stress": sim.read("stress")[:, [0, 1, 3]]}


def err(a, b):
    """(error, kind): normwise relative, or RMS absolute where b is zero."""
    b = np.asarray(b, np.float64)
    if np.linalg.norm(b) == 0.0:
        d = np.asarray(a, np.float64) - b
        return float(np.sqrt(np.mean(d * d))), "abs"
    return rel(a, b), "rel"


def compare(name, gpu, f32, f64):
    (e_gpu, kind), (e_ref, _) = err(gpu, f64), err(f32, f64)
    assert e_gpu <= max(3.0 * e_ref, FLOOR), (name, e_gpu, e_ref)
    return e_gpu, e_ref, kind


def record(config, gpu, f32, f64):
    row = {"config": config}
    for k in gpu:
        row[k] = compare((config, k), gpu[k], f32[k], f64[k])
    TABLE.append(row)


def run_pair(builder, steps, **kw):
    gs, g, _ = builder(D, sim_steps=steps, **kw)
    o32, _, _ = builder(O, sim_steps=steps, **kw)
    o64, _, _ = builder(O, sim_steps=steps, dtype=np.float64, **kw)
    sim = gs.simulation(g, reinit=True)
    gs._upload(sim)
    sim.initialize()
    sim.step(steps)
    for i in range(steps):
        o32.step(i, g, reinit=True)
        o64.step(i, g, reinit=True)
    out = gpu_fields(sim)
    sim.close()
    return out, fields_of(o32.mesh.particles[0]), fields_of(o64.mesh.particles[0])


def test_fp64_plain_small(built):
    """The reference's CPU case, full size: 144 particles, 1000 steps."""
    gpu, f32, f64 = run_pair(workloads.plain_small, 1000)
    record("plain 10x10, 144 particles, 1000 steps", gpu, f32, f64)


@pytest.mark.parametrize("scheme", ["usf", "usl"])
def test_fp64_scaleup(built, scheme):
    gpu, f32, f64 = run_pair(workloads.plain_scaleup, 100, n=64, scheme=scheme)
    record(f"scale-up {scheme.upper()} at 64x64 (8,192 particles), 100 steps", gpu, f32, f64)


def test_fp64_mixed(built):
    gpu, f32, f64 = run_pair(workloads.mixed_large, 100, n=64)
    record("mixed elastic + Newtonian USL at 64x64, 100 steps", gpu, f32, f64)


def test_fp64_differentiation(built):
    """Forward fields, and the adjoint dL/dE against float64 autograd."""
    torch = pytest.importorskip("torch")
    from oracle import mpm_torch as T
    # dt 5e-5 (CFL ~0.07 at this mesh) so the 200 steps move the particles by
    # ~5e-4 m, well above the float32 resolution of the positions
    n, steps, dt = 32, 200, 5e-5
    gpu, f32, f64 = run_pair(workloads.differentiation, steps, n=n, dt=dt)
    row_name = f"differentiation at 32x32 ({len(gpu['velocity'])} particles), {steps} steps"
    record(row_name, gpu, f32, f64)
    # gradient of L = mean |x_end - x_target|^2, target from another E field
    ts, tg, _ = workloads.differentiation(D, n=n, sim_steps=steps, dt=dt, seed=202)
    tsim = ts.simulation(tg, reinit=True)
    ts._upload(tsim)
    tsim.initialize()
    tsim.step(steps)
    target = tsim.read("loc").astype(np.float64)
    tsim.close()
    gs, g, info = workloads.differentiation(D, n=n, sim_steps=steps, dt=dt)
    sim = gs.simulation(g, reinit=True)
    gs._upload(sim)
    sim.initialize()
    sim.record(steps, 50)
    npart = info["np"]
    seed = (2.0 / npart * (sim.read("loc") - target)).astype(np.float32)
    got = sim.adjoint(seed, want=("youngs_modulus",))["youngs_modulus"]
    sim.close()
    grads = {}
    for dt_ in (torch.float32, torch.float64):
        npd = np.float32 if dt_ == torch.float32 else np.float64
        o, og, oi = workloads.differentiation(O, n=n, sim_steps=steps, dt=dt, dtype=npd)
        tsim_, st0 = T.from_solver(o, og, dtype=dt_)
        Et = torch.tensor(oi["E"], dtype=dt_, requires_grad=True)
        end = tsim_.run(dict(st0), steps, E=Et)
        L = ((end["x"] - torch.tensor(target, dtype=dt_)) ** 2).sum(1).mean()
        L.backward()
        grads[dt_] = Et.grad.numpy()
    e_gpu = rel(got, grads[torch.float64])
    e_ref = rel(grads[torch.float32], grads[torch.float64])
    assert rel(got, grads[torch.float32]) < 1e-3
    assert e_gpu <= max(3.0 * e_ref, 1e-3), (e_gpu, e_ref)
    TABLE[-1]["dL/dE"] = (e_gpu, e_ref, "rel")


def test_fp64_batch_members(built):
    """Three batch members advanced together in one batch, 300 steps."""
    specs = workloads.batch_specs(nsims=3, seed=3, sides=(24, 48))
    steps = 300
    sims, gs_ = [], []
    for sp in specs:
        solver, g, _ = workloads.batch_member(D, sp, sim_steps=steps)
        sim = solver.simulation(g, reinit=True)
        solver._upload(sim)
        sim.initialize()
        sims.append(sim)
        gs_.append(g)
    batch = D.Batch(sims)
    batch.step(steps)
    worst = {}
    for sp, sim, g in zip(specs, sims, gs_):
        o32, _, _ = workloads.batch_member(O, sp, sim_steps=steps)
        o64, _, _ = workloads.batch_member(O, sp, sim_steps=steps, dtype=np.float64)
        for i in range(steps):
            o32.step(i, g, reinit=True)
            o64.step(i, g, reinit=True)
        gpu = gpu_fields(sim)
        f32 = fields_of(o32.mesh.particles[0])
        f64 = fields_of(o64.mesh.particles[0])
        for k in gpu:
            e = compare((sp["side"], k), gpu[k], f32[k], f64[k])
            if k not in worst or e[0] > worst[k][0]:
                worst[k] = e
    batch.close()
    for sim in sims:
        sim.close()
    TABLE.append(dict({"config": f"batch members (sides {[s['side'] for s in specs]}), "
                                 f"{steps} steps, worst member"}, **worst))
