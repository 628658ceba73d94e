"""Benchmark of the explicit MPM step and its adjoint on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload batch|plain] [--nsims 512] [--checkpoint-steps 100]

Default workload (``batch``): the batching configuration -- 512 independent
2-D USF simulations of uneven size (mesh side uniform in {32..256}, 4 Gauss-
point particles per cell over a seeded random rectangle covering 20-60% of
the domain, E log-uniform in [1e5, 1e8], nu in [0.2, 0.35], rho 1500,
gravity, bottom fixed, dt from CFL 0.3; 19.6M particles in total), 1000
steps, float32.  The headline ``value`` is batched forward + adjoint
particle-steps/s: one checkpointed batched forward run (mpm_batch_record,
checkpoints every 100 steps) plus the batched adjoint w.r.t. each
simulation's E (mpm_batch_adjoint) of L = mean |x_end - x_target|^2, timed
with CUDA events after one untimed warm-up iteration.  Beside it: the same
batch forward only, and the plain path -- each simulation advanced alone by
mpm_step, one after another -- the denominator of the batched / plain
ratios in ``components``.  The plain 2-D scale-up (1024^2 mesh, 2.1M
particles, 500 steps, USF and USL) is measured too and gives the roofline of
the plain top kernel; the 4096^2 elastic + Newtonian run (16.8M particles,
200 USL steps) and the 256^2 differentiation run (2000 steps) are timed
beside them.

``--impl reference`` times the CPU restatement of the reference step and its
autograd gradient (the reference itself is JAX, not installed) on a sample of
the same simulations with every host core (one process per core).  Under
torchrun each rank runs an independent replica (weak scaling) and rank 0
prints.
"""
from __future__ import annotations

import argparse
import json
import os
import platform
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "particle-steps/s: batched fwd+adjoint vs plain fwd, 1 GB300, rel err ≤1e-5"
UNIT = "particle-steps/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="batch", choices=["batch", "plain"])
    ap.add_argument("--nsims", type=int, default=512)
    ap.add_argument("--checkpoint-steps", type=int, default=100)
    ap.add_argument("--scheme", default="usf", choices=["usf", "usl"])
    ap.add_argument("--n", type=int, default=1024, help="mesh side of the plain scale-up")
    ap.add_argument("--plain-steps", type=int, default=500)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-plain-path", action="store_true",
                    help="skip timing each simulation alone (the ratio's denominator)")
    ap.add_argument("--phase-steps", type=int, default=20)
    ap.add_argument("--mixed-steps", type=int, default=200,
                    help="steps of the 4096^2 elastic + Newtonian workload (0 skips it)")
    ap.add_argument("--diff-steps", type=int, default=2000,
                    help="steps of the differentiation workload (0 skips it)")
    ap.add_argument("--cpu-configs", action="store_true",
                    help="CPU only: time the float32 restatements of the reference step on a "
                         "bounded sample of each configuration, one core, and print one JSON line")
    return ap.parse_args()


def max_over_ranks(value, world, device="cpu"):
    """The largest of every rank's ``value`` (the job's time is its slowest
    rank's); ``value`` itself when there is one rank."""
    if world <= 1:
        return value
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group(backend="nccl" if args.impl == "ours" else "gloo")
    return world, rank, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons, power = [], [], set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
                power.append(float(f[3]))
            except ValueError:
                continue
            for name, val in zip(names, f[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "power_w_max": max(power) if power else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def measured_peak():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def phase_bytes(np_, nn, scheme):
    """Algorithmic bytes per launch of each phase (unique float32 traffic)."""
    if scheme == "usf":
        return {"nodal_kinematics": 20 * np_ + 12 * nn,
                "forces": 80 * np_ + 28 * nn,
                "particle_kinematics": 32 * np_ + 16 * nn}
    return {"nodal_kinematics": 20 * np_ + 12 * nn,
            "forces": 28 * np_ + 28 * nn,
            "particle_kinematics": 104 * np_ + 16 * nn}


# ---------------------------------------------------------------------------
# CPU arms: the NumPy / torch float32 restatements of the reference step
# ---------------------------------------------------------------------------
def _cpu_fwd_adj_member(args):
    """Forward + autograd backward of `steps` steps of one batch member with
    the float32 torch restatement; returns (particle-steps, seconds)."""
    k, steps, seed_specs = args
    import torch
    torch.set_num_threads(1)
    from diffmpm_gb300 import workloads
    from oracle import mpm_oracle as O
    from oracle import mpm_torch as T
    if steps == 0:                       # pool warm-up: imports only
        return 0, 0.0
    spec = workloads.batch_specs(**seed_specs)[k]
    o, g, info = workloads.batch_member(O, spec, sim_steps=steps)
    sim, st0 = T.from_solver(o, g, dtype=torch.float32)
    n = info["np"]
    t0 = time.perf_counter()
    E = torch.tensor(spec["E"], dtype=torch.float32, requires_grad=True)
    end = sim.run(dict(st0), steps, E=E.expand(n))
    L = ((end["x"] - st0["x"] - 1e-4) ** 2).sum(1).mean()
    L.backward()
    return n * steps, time.perf_counter() - t0


def cpu_fwd_adj(members, steps, workers, seed_specs=None):
    """Particle-steps/s of forward + adjoint on the CPU over `members`, timed
    by the wall clock around the whole pool's work (after a warm-up task on
    every worker, so that process start-up and imports are outside it).
    Members go largest first to keep the workers evenly loaded."""
    import multiprocessing as mp
    from diffmpm_gb300 import workloads
    specs = workloads.batch_specs(**(seed_specs or {}))
    order = sorted(members, key=lambda k: -specs[k]["np"])
    jobs = [(k, steps, seed_specs or {}) for k in order]
    if workers > 1:
        with mp.get_context("spawn").Pool(workers) as pool:
            pool.map(_cpu_fwd_adj_member, [(0, 0, {})] * workers, chunksize=1)
            t0 = time.perf_counter()
            res = pool.map(_cpu_fwd_adj_member, jobs, chunksize=1)
            wall = time.perf_counter() - t0
    else:
        t0 = time.perf_counter()
        res = [_cpu_fwd_adj_member(j) for j in jobs]
        wall = time.perf_counter() - t0
    ps = sum(r[0] for r in res)
    return ps / wall, ps, wall


def cpu_sample_members(nsims, limit_particles):
    """The first batch members whose particle counts add up to `limit_particles`."""
    from diffmpm_gb300 import workloads
    specs = workloads.batch_specs(nsims=nsims)
    out, tot = [], 0
    for k, sp in enumerate(specs):
        if tot + sp["np"] > limit_particles and out:
            break
        out.append(k)
        tot += sp["np"]
    return out, tot


# The CPU sample shared by the `cpu_baseline` leg of the GPU arm and by the
# reference arm: the first batch members holding about 40,000 particles per
# host core, forward + adjoint, one process per core.
CPU_PARTICLES_PER_CORE = 40000


def cpu_sample(nsims, workers):
    members, tot = cpu_sample_members(nsims, CPU_PARTICLES_PER_CORE * workers)
    return members, tot


def cpu_sample_text(members, tot, steps):
    return (f"{steps} steps of batch members {members[0]}..{members[-1]} ({tot} particles), "
            f"float32 torch restatement of the reference step, forward + autograd adjoint "
            f"w.r.t. each simulation's E, one process per core, wall-clock time of the pool "
            f"(JAX is not installed)")


def run_reference(args, world, rank):
    if rank != 0:
        return
    workers = os.cpu_count() or 1
    steps = args.steps
    members, tot = cpu_sample(args.nsims, workers)
    for _ in range(max(0, min(args.warmup, 1))):
        cpu_fwd_adj(members[:workers], 2, workers)
    v, ps, wall = cpu_fwd_adj(members, steps, workers)
    sample = cpu_sample_text(members, tot, steps)
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * wall / steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": "batch_fwd_adjoint", "sims": args.nsims, "steps": steps,
                   "sample_members": [members[0], members[-1]], "sample_particles": tot,
                   "sample": sample},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": workers, "kind": "port",
                         "sample": sample},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


def run_cpu_configs():
    """Per-configuration CPU figures beside the GPU ones: the float32 NumPy
    restatement of the reference step (forward, ``np.add.at`` scatters in
    particle order) on a bounded sample of steps of each configuration at its
    full size, and the float32 torch restatement's forward + autograd adjoint
    w.r.t. the per-particle E on the differentiation configuration; one
    process on one core."""
    import torch
    from diffmpm_gb300 import workloads
    from oracle import mpm_oracle as O
    from oracle import mpm_torch as T
    torch.set_num_threads(1)
    out = {}

    def forward(name, builder, steps, **kw):
        solver, g, info = builder(O, sim_steps=steps, **kw)
        t0 = time.perf_counter()
        for i in range(steps):
            solver.step(i, g)
        sec = time.perf_counter() - t0
        out[name] = {"what": "forward, NumPy float32", "particles": info["np"], "steps": steps,
                     "seconds": sec, "value": info["np"] * steps / sec}

    forward("plain_small_10x10_usf", workloads.plain_small, 1000)
    forward("plain_scaleup_1024_usf", workloads.plain_scaleup, 2, n=1024, scheme="usf")
    forward("plain_scaleup_1024_usl", workloads.plain_scaleup, 2, n=1024, scheme="usl")
    forward("mixed_large_4096_usl", workloads.mixed_large, 1)
    forward("differentiation_256_usf", workloads.differentiation, 20)
    steps = 20
    o, g, info = workloads.differentiation(O, sim_steps=steps)
    sim, st0 = T.from_solver(o, g, dtype=torch.float32)
    t0 = time.perf_counter()
    E = torch.tensor(info["E"], dtype=torch.float32, requires_grad=True)
    end = sim.run(dict(st0), steps, E=E)
    ((end["x"] - st0["x"] - 1e-4) ** 2).sum(1).mean().backward()
    sec = time.perf_counter() - t0
    out["differentiation_256_usf_fwd_adjoint"] = {
        "what": "forward + autograd adjoint w.r.t. E, torch float32", "particles": info["np"],
        "steps": steps, "seconds": sec, "value": info["np"] * steps / sec}
    print(json.dumps({"impl": "cpu-configs", "unit": UNIT, "cores": 1, "kind": "port",
                      "host": platform.machine(), "configs": out}), flush=True)


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
def build_batch(D, workloads, nsims, steps):
    specs = workloads.batch_specs(nsims=nsims)
    members = []
    for sp in specs:
        solver, g, info = workloads.batch_member(D, sp, sim_steps=steps)
        sim = solver.simulation(g, reinit=True)
        solver._upload(sim)
        sim.initialize()
        members.append((solver, sim, g))
    return specs, members


def reset_batch(members):
    for solver, sim, g in members:
        solver._upload(sim)
        sim.initialize()


def plain_scaleup(args, D, workloads, torch):
    """The plain 2-D scale-up: device-timed forward, per-phase kernel times and
    the roofline of the top kernel."""
    solver, g, info = workloads.plain_scaleup(D, n=args.n, scheme=args.scheme,
                                              sim_steps=args.plain_steps)
    np_, nn = info["np"], (args.n + 1) ** 2
    sim = solver.simulation(g, reinit=True)
    solver._upload(sim)
    sim.initialize()
    sim.set_block_steps(100)
    sim.step(max(args.warmup, 3))
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    sim.step(args.plain_steps)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    tot = sim.time_phases(args.phase_steps)
    avg = {k: v / args.phase_steps for k, v in tot.items()}
    top = max(avg, key=avg.get)
    pb = phase_bytes(np_, nn, args.scheme)
    peak, peak_kind = measured_peak()
    achieved = pb[top] / (avg[top] / 1000.0) / 1e9
    traffic = None   # DRAM bytes of one launch from the committed ncu summary
    tf = ROOT / "profiles" / f"k_{top}_plain_scaleup_{args.scheme}.md"
    if tf.exists():
        for line in tf.read_text().splitlines():
            if line.startswith("dram bytes per launch:"):
                traffic = int(line.split(":")[1])
    out = {
        "workload": f"plain_scaleup_{args.scheme}", "mesh": f"{args.n}x{args.n}", "particles": np_,
        "steps": args.plain_steps, "value": np_ * args.plain_steps / (ms / 1000.0),
        "ms_per_step": ms / args.plain_steps, "phase_ms": avg,
        "step_roofline_frac": (workloads.particle_steps_bytes(np_, nn) * args.plain_steps
                               / (ms / 1000.0) / 1e9) / peak,
    }
    roof = {"bound": "hbm", "kernel": top, "workload": out["workload"], "achieved": achieved,
            "peak": peak, "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak,
            "traffic": traffic, "algorithmic_bytes": pb[top]}
    sim.close()
    return out, roof


def mixed_large(args, D, workloads, torch):
    """The large mixed-material workload: 4096^2 mesh, 16,777,216 particles in
    a LinearElastic and a Newtonian block, USL, dt 2e-7; device-timed steps
    in graphs of 100 and per-phase kernel times."""
    K = args.mixed_steps
    solver, g, info = workloads.mixed_large(D, sim_steps=K)
    np_, nn = info["np"], (info["n"] + 1) ** 2
    sim = solver.simulation(g, reinit=True)
    solver._upload(sim)
    sim.initialize()
    sim.set_block_steps(100)
    sim.step(max(args.warmup, 3))
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    sim.step(K)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    tot = sim.time_phases(args.phase_steps)
    peak, _ = measured_peak()
    out = {"workload": "mixed_large_usl", "mesh": f"{info['n']}x{info['n']}", "particles": np_,
           "steps": K, "value": np_ * K / (ms / 1000.0), "ms_per_step": ms / K,
           "phase_ms": {k: v / args.phase_steps for k, v in tot.items()},
           "step_roofline_frac": (workloads.particle_steps_bytes(np_, nn) * K
                                  / (ms / 1000.0) / 1e9) / peak}
    sim.close()
    return out


def differentiation(args, D, workloads, torch):
    """The differentiation workload: 256^2 mesh, 125,664 particles with a
    seeded log-normal E field, 2000 USF steps; loss = mean |x_end - x_target|^2
    against a forward run from another seeded field; gradient w.r.t. the
    per-particle E through the checkpointed adjoint (checkpoints every 100)."""
    K = args.diff_steps
    ts, tg, _ = workloads.differentiation(D, sim_steps=K, seed=202)
    tsim = ts.simulation(tg, reinit=True)
    ts._upload(tsim)
    tsim.initialize()
    tsim.step(K)
    target = tsim.read("loc")
    tsim.close()
    solver, g, info = workloads.differentiation(D, sim_steps=K, seed=101)
    sim = solver.simulation(g, reinit=True)
    n = info["np"]

    def reset():
        solver._upload(sim)
        sim.initialize()

    def seed():
        x = sim.read("loc")
        d = x.astype(np.float64) - target
        return (2.0 / n * d).astype(np.float32), float((d * d).sum(1).mean())

    ckpt = min(args.checkpoint_steps, K)
    reset()
    sim.record(K, ckpt)
    sim.adjoint(seed()[0], want=("youngs_modulus",))
    e = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    reset()
    torch.cuda.synchronize()
    e[0].record()
    sim.record(K, ckpt)
    e[1].record()
    torch.cuda.synchronize()
    sd, loss = seed()
    e[2].record()
    gr = sim.adjoint(sd, want=("youngs_modulus",))["youngs_modulus"]
    e[3].record()
    torch.cuda.synchronize()
    rec_ms, adj_ms = e[0].elapsed_time(e[1]), e[2].elapsed_time(e[3])
    reset()
    torch.cuda.synchronize()
    e[0].record()
    sim.step(K)
    e[1].record()
    torch.cuda.synchronize()
    fwd_ms = e[0].elapsed_time(e[1])
    sim.close()
    ps = n * K
    return {"workload": "differentiation", "mesh": "256x256", "particles": n, "steps": K,
            "checkpoint_steps": ckpt, "loss": loss,
            "dLdE_norm": float(np.linalg.norm(gr.astype(np.float64))),
            "fwd_adjoint": ps / ((rec_ms + adj_ms) / 1000.0), "fwd": ps / (fwd_ms / 1000.0),
            "record_ms": rec_ms, "adjoint_ms": adj_ms, "fwd_ms": fwd_ms}


def run_ours(args, world, rank, local):
    import torch
    torch.cuda.set_device(local)
    import diffmpm_gb300 as D
    from diffmpm_gb300 import workloads

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    def ev():
        return torch.cuda.Event(enable_timing=True)

    K = args.steps
    specs, members = build_batch(D, workloads, args.nsims, K)
    sims = [m[1] for m in members]
    npart = sum(sp["np"] for sp in specs)
    nnode = sum((sp["side"] + 1) ** 2 for sp in specs)
    batch = D.Batch(sims)
    _, ntiles = batch.size()
    tuning = batch.autotune(trial_steps=100)
    block = tuning["block_steps"]
    ckpt = min(args.checkpoint_steps, K)
    x0 = [sim.read("loc") for sim in sims]
    targets = [x + 1e-4 for x in x0]

    def seeds_for():
        out = []
        for sim, tgt in zip(sims, targets):
            x = sim.read("loc")
            out.append((2.0 / len(x) * (x - tgt)).astype(np.float32))
        return out

    # warm-up: W forward steps, then one full record + adjoint (allocations,
    # graph capture), then back to the initial state
    batch.step(max(args.warmup, 3))
    reset_batch(members)
    batch.record(K, ckpt)
    batch.adjoint(seeds_for(), want=("youngs_modulus",))
    reset_batch(members)
    torch.cuda.synchronize()
    barrier()

    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    # timed: batched forward + adjoint (an NVTX range "timed" for profilers)
    e0, e1, e2, e3 = ev(), ev(), ev(), ev()
    torch.cuda.nvtx.range_push("timed")
    e0.record()
    batch.record(K, ckpt)
    e1.record()
    torch.cuda.synchronize()
    seeds = seeds_for()
    e2.record()
    grads = batch.adjoint(seeds, want=("youngs_modulus",))
    e3.record()
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    rec_ms, adj_ms = e0.elapsed_time(e1), e2.elapsed_time(e3)
    fa_ms = max_over_ranks(rec_ms + adj_ms, world, device="cuda")
    dLdE = [float(g["youngs_modulus"].astype(np.float64).sum()) for g in grads]
    # batched forward only
    reset_batch(members)
    torch.cuda.synchronize()
    e0.record()
    batch.step(K)
    e1.record()
    torch.cuda.synchronize()
    fwd_ms = e0.elapsed_time(e1)
    clk = clocks.stop()
    counters = {"resorts": sum(s.counters()["resorts"] for s in sims),
                "rollbacks": sum(s.counters()["rollbacks"] for s in sims)}

    # end to end through the public API with host buffers: the initial states
    # of every member from pinned host memory (whole-batch writes and a
    # restart), record, positions back, adjoint with host seeds, gradients back
    def pinned(a):
        t = torch.empty(a.size, dtype=torch.float32, pin_memory=True).numpy()
        t[:] = a.reshape(-1)
        return t

    init = {}
    for name in ("loc", "velocity", "stress", "strain", "density", "volumetric_strain_centroid"):
        parts = []
        for solver, sim, g in members:
            p = solver.mesh.particles[0]
            v = {"loc": p.loc, "velocity": p.velocity, "stress": p.stress, "strain": p.strain,
                 "density": p.density,
                 "volumetric_strain_centroid": p.volumetric_strain_centroid}[name]
            parts.append(np.asarray(v, np.float32).reshape(-1))
        init[name] = pinned(np.concatenate(parts))
    node_v0 = pinned(np.concatenate([np.asarray(solver.mesh.elements.nodes.velocity, np.float32)
                                     .reshape(-1) for solver, sim, g in members]))
    target_flat = np.concatenate([t.reshape(-1) for t in targets]).astype(np.float32)
    scale = np.concatenate([np.full(2 * len(t), 2.0 / len(t), np.float32) for t in targets])
    loc_out = pinned(np.zeros(target_flat.size, np.float32))

    def e2e_upload():
        for name, arr in init.items():
            batch.write(name, arr)
        batch.write_nodal("velocity", node_v0)
        batch.restart()

    e2e_upload()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e2e_upload()
    t1 = time.perf_counter()
    batch.record(K, ckpt)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    xs = batch.read("loc", out=loc_out)
    seeds = batch.split("loc", scale * (xs - target_flat))
    t3 = time.perf_counter()
    grads = batch.adjoint(seeds, want=("youngs_modulus",))
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    e2e_parts = {"upload_s": t1 - t0, "record_s": t2 - t1, "seeds_s": t3 - t2,
                 "adjoint_s": e2e_s - (t3 - t0)}
    h2d = npart * (2 + 2 + 6 + 6 + 1 + 1) * 4 + nnode * 2 * 4 + sum(s.nbytes for s in seeds)
    d2h = npart * 2 * 4 + sum(g["youngs_modulus"].nbytes for g in grads)

    # plain path: each simulation alone, one after another
    plain_ms = None
    if not args.no_plain_path:
        batch.close()
        reset_batch(members)
        for sim in sims:
            sim.set_block_steps(100)
            sim.step(2)
        reset_batch(members)
        torch.cuda.synchronize()
        e0.record()
        for sim in sims:
            sim.step(K)
        e1.record()
        torch.cuda.synchronize()
        plain_ms = e0.elapsed_time(e1)
    for sim in sims:
        sim.close()
    del members, sims

    plain, roof = plain_scaleup(args, D, workloads, torch)
    # the scale-up configuration is run with both schemes; the USL line adds
    # its own top-kernel roofline for reference
    plain_usl, roof_usl = plain_scaleup(argparse.Namespace(**dict(vars(args), scheme="usl")), D,
                                        workloads, torch)
    plain_usl["roofline"] = roof_usl
    mixed = mixed_large(args, D, workloads, torch) if args.mixed_steps > 0 else None
    diff = differentiation(args, D, workloads, torch) if args.diff_steps > 0 else None

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        workers = os.cpu_count() or 1
        mem, tot = cpu_sample(args.nsims, workers)
        csteps = min(K, 20)
        v, ps, wall = cpu_fwd_adj(mem, csteps, workers)
        cpu = {"value": v, "unit": UNIT, "cores": workers, "kind": "port",
               "sample": cpu_sample_text(mem, tot, csteps)}

    ps = npart * K
    value = world * ps / (fa_ms / 1000.0)
    # kernels of ours launched in the timed region (record + adjoint), as
    # the code issues them (a 100-step run of this configuration counts
    # 3676; ncu's launch list of the same region counted 3166 before the
    # adjoint arrays were zeroed by one gather per simulation, 512 more):
    # record: 4 step kernels per step (empty tiles' nodes, nodal kinematics,
    #   forces, G2P); per block a counter advance, the tile split and records
    #   (4), the snapshot (chunk table + copy) and the status gather; per
    #   segment a checkpoint (chunk table + copy);
    # adjoint: per segment restore (2), status, epoch copy (2), tape tables
    #   (3), tile split and records (4), status and the re-run check (2);
    #   per re-run step 2 tape copies, the 4 step kernels and a counter
    #   advance; per reverse step the argument table and 4 passes; per
    #   simulation the read of its positions for the seeds, the zeroing and
    #   seed gathers and the gradient out (4); the final restore and status
    #   (3);
    # re-sorts: 21 kernels each (counted over the record and the forward
    #   alone: halved).
    nblk = (K + block - 1) // block
    launches = (4 * K + nblk * 8 + nseg_count(K, ckpt) * 2
                + nseg_count(K, ckpt) * 15 + K * (2 + 4 + 1) + K * 5 + 4 * args.nsims + 3
                + 21 * counters["resorts"] // 2)
    if rank == 0:
        print(json.dumps({
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K,
            "warmup": args.warmup, "ms_per_step": fa_ms / K, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "batch_fwd_adjoint", "sims": args.nsims, "particles": npart,
                       "nodes": nnode, "tiles_per_launch": ntiles, "steps": K,
                       "checkpoint_steps": ckpt, "block_steps": block,
                       "tuning": {k: tuning[k] for k in ("block_steps", "resort_every", "nk_ctas",
                                                         "g2p_ctas", "forces_lpc", "ms_per_step",
                                                         "from_cache")},
                       "domain_m": 0.05,
                       "dt": "CFL 0.3 per simulation", "scheme": "usf",
                       "loss": "mean |x_end - x_target|^2 per simulation, grad w.r.t. its E",
                       "l2": "inputs larger than L2 (~2 GB of particle state)",
                       "parallelism": f"replicas x{world}" if world > 1 else "single GPU"},
            "components": {
                "batch_fwd_adjoint": value / world,
                "batch_fwd": ps / (fwd_ms / 1000.0),
                "plain_fwd": ps / (plain_ms / 1000.0) if plain_ms else None,
                "ratio_fwd_adjoint_vs_plain_fwd": (plain_ms / fa_ms) if plain_ms else None,
                "ratio_batch_fwd_vs_plain_fwd": (plain_ms / fwd_ms) if plain_ms else None,
                "record_ms": rec_ms, "adjoint_ms": adj_ms, "batch_fwd_ms": fwd_ms,
                "plain_fwd_ms": plain_ms},
            "dLdE_first_sims": dLdE[:4],
            "e2e": {"value": world * ps / e2e_s, "unit": UNIT, "h2d_bytes_per_step": h2d / K,
                    "d2h_bytes_per_step": d2h / K,
                    "what": "whole-batch upload of all initial states from pinned host memory + "
                            "restart + batched record + positions to host + adjoint with host "
                            "seeds + gradients to host", "parts": e2e_parts},
            "gpu_launches": launches,
            "roofline": roof,
            "plain_scaleup": plain,
            "plain_scaleup_usl": plain_usl,
            "mixed_large": mixed,
            "differentiation": diff,
            "clocks": clk,
            "counters": counters,
            "cpu_baseline": cpu,
        }), flush=True)


def run_ours_plain(args, world, rank, local):
    """``--workload plain``: the plain scale-up alone (a short run for profiling)."""
    import torch
    torch.cuda.set_device(local)
    import diffmpm_gb300 as D
    from diffmpm_gb300 import workloads
    args.plain_steps = args.steps
    plain, roof = plain_scaleup(args, D, workloads, torch)
    if rank == 0:
        print(json.dumps({
            "metric": METRIC, "value": world * plain["value"], "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": plain["ms_per_step"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": {"workload": plain["workload"], "mesh": plain["mesh"],
                                            "particles": plain["particles"]},
            "roofline": roof, "plain_scaleup": plain}), flush=True)


def nseg_count(steps, ckpt):
    """Checkpoint segments of a recording of `steps` steps."""
    return (steps + ckpt - 1) // ckpt


def main():
    args = parse()
    if args.cpu_configs:
        run_cpu_configs()
        return
    world, rank, local = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, world, rank)
    elif args.workload == "plain":
        run_ours_plain(args, world, rank, local)
    else:
        run_ours(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
