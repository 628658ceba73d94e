"""Benchmark of the explicit MPM step on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload: the plain 2-D scale-up configuration -- 1024 x 1024 Q4 mesh, 4
jittered Gauss-point particles per cell over x in [0, 0.5] (2,097,152
particles), LinearElastic E=1e6 nu=0.25 rho=2000, gravity, roller walls and
fixed bottom, dt=1e-6, USF (``--scheme usl`` for USL), float32.  A step is one
explicit MPM step of the whole population.  The state (~190 MB) is larger than
the 129 MB L2.

Our arm prints one JSON line: device-timed particle-steps/s (``value``), an
end-to-end number through the public API with host buffers (``e2e``), the
roofline of the dominant kernel from CUDA-event timing of each phase, clocks
sampled during the timed region, and a CPU baseline (the NumPy restatement of
the reference step, one core, on a bounded sample).  ``--impl reference``
times that CPU restatement alone (the reference itself is JAX, which is not
installed on these machines).  Under torchrun each rank runs an independent
replica (weak scaling) and rank 0 prints.
"""
from __future__ import annotations

import argparse
import json
import os
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
MESH_N = 1024


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=500)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--scheme", default="usf", choices=["usf", "usl"])
    ap.add_argument("--n", type=int, default=MESH_N)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--phase-steps", type=int, default=20)
    return ap.parse_args()


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        backend = "nccl" if args.impl == "ours" else "gloo"
        dist.init_process_group(backend=backend)
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


def cpu_baseline(n, scheme, steps=2):
    """The NumPy float32 restatement on the full workload, `steps` steps, one core."""
    from oracle import mpm_oracle as O
    from diffmpm_gb300 import workloads
    s, g, info = workloads.plain_scaleup(O, n=n, scheme=scheme, sim_steps=steps)
    t0 = time.perf_counter()
    for i in range(steps):
        s.step(i, g)
    dt = time.perf_counter() - t0
    return {"value": info["np"] * steps / dt, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"{steps} of the 500 steps of the full workload ({info['np']} particles), "
                      f"NumPy float32 restatement of the reference step"}


def run_reference(args, world, rank):
    """CPU restatement of the reference step (the reference is JAX, not installed)."""
    if rank != 0:
        return
    from oracle import mpm_oracle as O
    from diffmpm_gb300 import workloads
    rows = max(8, args.n // 8)
    s, g, info = workloads.plain_scaleup(O, n=args.n, scheme=args.scheme,
                                         sim_steps=args.steps + args.warmup, rows=rows)
    for i in range(args.warmup):
        s.step(i, g)
    t0 = time.perf_counter()
    for i in range(args.warmup, args.warmup + args.steps):
        s.step(i, g)
    el = time.perf_counter() - t0
    v = info["np"] * args.steps / el
    sample = (f"rows [0, {rows}) of the {args.n}x{args.n} workload ({info['np']} particles) per step, "
              f"NumPy float32 restatement of the reference step (JAX is not installed)")
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * el / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": f"plain_scaleup_{args.scheme}", "mesh": f"{args.n}x{args.n}",
                   "particles": info["np"], "sample": sample},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": 1, "kind": "port", "sample": sample},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


def run_ours(args, world, rank, local):
    import torch
    torch.cuda.set_device(local)
    import diffmpm_gb300 as D
    from diffmpm_gb300 import workloads

    solver, g, info = workloads.plain_scaleup(D, n=args.n, scheme=args.scheme,
                                              sim_steps=args.steps)
    np_ = info["np"]
    nn = (args.n + 1) ** 2
    sim = solver.simulation(g, reinit=True)
    solver._upload(sim)
    sim.initialize()
    sim.set_block_steps(min(100, max(1, args.steps)))
    stream = torch.cuda.current_stream()

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    # warm-up (captures the step graphs)
    sim.step(max(args.warmup, 3))
    torch.cuda.synchronize()
    barrier()
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    sim.step(args.steps)
    e1.record(stream)
    torch.cuda.synchronize()
    barrier()
    clk = clocks.stop()
    ms = e0.elapsed_time(e1)
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    value = world * np_ * args.steps / (ms / 1000.0)
    counters = sim.counters()

    # per-phase kernel time: CUDA events recorded between back-to-back launches
    # of the phase kernels on the launching stream
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

    # end to end through the public API with host buffers: upload, set-up,
    # K steps, read back loc/velocity/stress/strain (solve_jit's outputs)
    host = {k: np.ascontiguousarray(v) for k, v in {
        "loc": solver.mesh.particles[0].loc.reshape(-1, 2),
        "velocity": solver.mesh.particles[0].velocity.reshape(-1, 2)}.items()}
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    solver._upload(sim)
    sim.initialize()
    sim.step(args.steps)
    outs = {k: sim.read(k) for k in ("loc", "velocity", "stress", "strain")}
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    h2d = np_ * (2 + 2 + 6 + 6 + 1 + 1 + 1) * 4 + nn * 2 * 4
    d2h = sum(v.nbytes for v in outs.values())
    del host

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(args.n, args.scheme)

    if rank == 0:
        print(json.dumps({
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": f"plain_scaleup_{args.scheme}", "mesh": f"{args.n}x{args.n}",
                       "particles": np_, "nodes": nn, "dt": 1e-6,
                       "l2": "inputs larger than L2 (~190 MB resident state)",
                       "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
                       "block_steps": min(100, max(1, args.steps))},
            "e2e": {"value": world * np_ * args.steps / e2e_s, "unit": UNIT,
                    "h2d_bytes_per_step": h2d / args.steps, "d2h_bytes_per_step": d2h / args.steps,
                    "what": "upload + set-up + K steps + read of loc/velocity/stress/strain, host arrays"},
            "gpu_launches": 3 * args.steps + 9 * counters.get("resorts", 0),
            "phase_ms": avg,
            "roofline": {"bound": "hbm", "kernel": top, "achieved": achieved, "peak": peak,
                         "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": traffic, "algorithmic_bytes": pb[top]},
            "step_roofline_frac": (workloads.particle_steps_bytes(np_, nn) * args.steps
                                   / (ms / 1000.0) / 1e9) / peak,
            "clocks": clk,
            "counters": counters,
            "cpu_baseline": cpu,
        }), flush=True)


def main():
    args = parse()
    world, rank, local = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_ours(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
