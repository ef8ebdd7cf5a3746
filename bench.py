#!/usr/bin/env python
"""Benchmark of the vortex-particle + panel induction step on one GB300.

Workload: the synthetic wake of ``fluxvortex_gb300.workloads.slab_wake`` at
2^20 (~1e6) particles, Winckelmans core sigma = 0.02c, plus the 4096
collocation points of a 64 x 64 wing grid.  One step =
  wake-on-collocation induction (4096 targets x N particles) +
  one VortexParticleField.advect_rk3 step with free wake and stretching
  (3 x [velocity sweep, position update, stretching sweep, strength update])
  + NaN guard + Pedrizzetti relaxation (Gaussian-erf vorticity sweep),
all resident in HBM.  Sweeps run FP32 with compensated accumulation; the
time integration is FP64.

Output: one JSON line (rank 0).  ``value`` = steps/s of the whole job
(device-timed, inputs resident); ``e2e`` = the same through the host-facing
API (particle state copied in from pinned host memory and the new state plus
the collocation velocities copied back every step); ``fp64_direct`` = the
same step with FP64 sweeps, timed on a target sample and scaled (all-pairs
cost is linear in the target count); ``cpu_baseline`` = the FP64 C oracle on
the host cores on a bounded target sample, scaled likewise.

``--impl reference`` times the reference's CPU path for this step (its
arithmetic restated in C + OpenMP, all host cores) on a bounded sample.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "VPM+panel steps/s at 1e6 particles: learned/FP32 vs FP64 direct @CL err<=1e-4"
UNIT = "steps/s"

# Algorithmic flop per (target, source) pair, counting + - * as 1, FMA as 2,
# sqrt / rsqrt / div / exp / erf as 1 ("Work per unit").
FLOP_PER_PAIR = {
    ("velocity", "winckelmans"): 30,
    ("stretch", "winckelmans"): 57,
    ("vorticity", "winckelmans"): 45,
    ("vorticity", "gaussianerf"): 55,
    ("velocity", "gaussianerf"): 40,
    ("stretch", "gaussianerf"): 67,
}
MODE_NAMES = {0: "velocity", 1: "stretch", 2: "velocity_stretch", 3: "jacobian", 4: "vorticity"}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--n", type=int, default=1 << 20, help="particles")
    p.add_argument("--precision", default="f32c", choices=["f32c", "f64"])
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-baselines", action="store_true")
    return p.parse_args()


# ---------------------------------------------------------------------------
def start_clock_sampler():
    path = tempfile.mktemp(prefix="clocks_", suffix=".csv")
    q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    try:
        f = open(path, "w")
        proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                 "-lms", "200"], stdout=f, stderr=subprocess.DEVNULL)
        return proc, f, path
    except (OSError, FileNotFoundError):
        return None, None, path


def stop_clock_sampler(handle, gpu_index=0):
    proc, f, path = handle
    if proc is None:
        return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
    proc.terminate()
    try:
        proc.wait(timeout=5)
    except subprocess.TimeoutExpired:
        proc.kill()
    f.close()
    sm, smax, reasons = [], [], set()
    names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
    for line in open(path):
        parts = [x.strip() for x in line.split(",")]
        if len(parts) < 9 or parts[0] != str(gpu_index):
            continue
        try:
            sm.append(float(parts[1]))
            smax.append(float(parts[2]))
        except ValueError:
            continue
        for nm, v in zip(names, parts[5:9]):
            if v.lower() == "active":
                reasons.add(nm)
    os.unlink(path)
    if not sm:
        return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
    loaded = [x for x in sm if x > 0.5 * max(sm)] or sm
    return {"sm_mhz": statistics.median(loaded), "sm_max_mhz": max(smax),
            "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
class Step:
    """The benchmarked step on one device (state resident in HBM)."""

    def __init__(self, n, precision, device):
        import torch
        from fluxvortex_gb300.particles import VortexParticleField
        from fluxvortex_gb300.workloads import slab_wake
        pos, gam, sig, colloc = slab_wake(n)
        self.host = dict(pos=pos, gamma=gam, sigma=sig, colloc=colloc)
        self.field = VortexParticleField(max_particles=n, nu=0.0, rlxf=0.3, kernel="winckelmans",
                                         precision=precision, device=device)
        self.field.add_particles_batch(pos, gam, sig)
        self.colloc = torch.as_tensor(colloc, device=device)
        self.u_colloc = torch.empty_like(self.colloc)
        self.u_inf = [10.0, 0.0, 0.0]
        self.dt = 0.02       # 0.2 chord per step at 10 m/s
        self.device = device

    def run(self):
        self.field._sweep(0, self.colloc, None, self.colloc.shape[0], self.u_colloc)
        self.field.advect_rk3(self.dt, self.u_inf, stretch=True, free_wake=True)


def sample_sweeps(field, n_t, precision, reps=1):
    """Times each sweep kind of one step on the first n_t particles as targets
    (all particles as sources); returns seconds per full step, scaled by
    N / n_t (the target count) -- exact for all-pairs work."""
    import torch
    from fluxvortex_gb300 import _capi
    n = field.np
    t = field._pos[:n_t]
    tg = field._gamma[:n_t]
    out = torch.empty((n_t, 3), dtype=torch.float64, device=field.device)
    old = field.precision
    field.precision = precision
    kinds = {"velocity": (_capi.PAIR_VELOCITY, None, "winckelmans"),
             "stretch": (_capi.PAIR_STRETCH, tg, "winckelmans"),
             "vorticity": (_capi.PAIR_VORTICITY, None, "gaussianerf")}
    sec = {}
    for name, (mode, tgm, kern) in kinds.items():
        field._sweep(mode, t, tgm, n_t, out, kernel=kern)          # warm-up
        torch.cuda.synchronize()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        for _ in range(reps):
            field._sweep(mode, t, tgm, n_t, out, kernel=kern)
        e.record()
        torch.cuda.synchronize()
        sec[name] = s.elapsed_time(e) / reps / 1e3
    field.precision = old
    full = n / n_t
    # 3 velocity + 3 stretching + 1 vorticity sweeps over all N targets, plus
    # the collocation sweep (4096 targets)
    return (3 * sec["velocity"] + 3 * sec["stretch"] + sec["vorticity"]) * full + \
        sec["velocity"] * 4096 / n_t


def cpu_oracle_step_seconds(host, n_t, threads=None):
    """FP64 C oracle (OpenMP) on n_t targets against all N sources for every
    sweep of the step; returns (seconds per full step, threads)."""
    import numpy as np
    from oracle import oracle as O
    if threads:
        O.set_num_threads(threads)
    pos, gam, sig = host["pos"], host["gamma"], host["sigma"]
    n = pos.shape[0]
    t, tg = pos[:n_t], gam[:n_t]
    t0 = time.perf_counter()
    O.velocity_from_particles(t, pos, gam, sig, "winckelmans")
    t_vel = time.perf_counter() - t0
    t0 = time.perf_counter()
    O.velocity_and_stretching(t, tg, pos, gam, sig, "winckelmans")
    t_vs = time.perf_counter() - t0
    t0 = time.perf_counter()
    O.jacobian_from_particles(t, tg, pos, gam, sig, "gaussianerf")
    t_j = time.perf_counter() - t0
    scale = n / n_t
    # step: 3 velocity + 3 stretching (a velocity+stretch pass bounds the
    # stretching pass) + 1 vorticity (Jacobian) + collocation (4096 targets)
    step = (3 * t_vel + 3 * t_vs + t_j) * scale + t_vel * 4096 / n_t
    return step, O.num_threads(), dict(velocity_s=t_vel, stretch_s=t_vs, jacobian_s=t_j,
                                       targets=n_t, sources=n)


# ---------------------------------------------------------------------------
def run_reference(args, rank, world):
    if rank != 0:
        return
    from fluxvortex_gb300.workloads import slab_wake
    pos, gam, sig, colloc = slab_wake(args.n)
    host = dict(pos=pos, gamma=gam, sigma=sig)
    cores = os.cpu_count() or 1
    n_t = max(16, int(64 * (1 << 20) / args.n))
    times = []
    for _ in range(args.warmup):
        cpu_oracle_step_seconds(host, max(4, n_t // 8), cores)
    for _ in range(args.steps):
        s, thr, detail = cpu_oracle_step_seconds(host, n_t, cores)
        times.append(s)
    step_s = statistics.median(times)
    v = 1.0 / step_s
    sample = (f"{n_t} targets x {args.n} sources per sweep kind (velocity, velocity+stretching, "
              f"Gaussian-erf Jacobian), scaled to the full step by N/targets")
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_s * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": f"slab wake, {args.n} particles + 4096 collocation points, "
                               "one RK3 free-wake step with stretching and relaxation"},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": thr, "kind": "port",
                         "sample": sample},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


def run_ours(args, rank, world):
    import torch
    import torch.distributed as dist
    from fluxvortex_gb300 import _capi

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    device = torch.device("cuda", local)
    lib = _capi.load()

    step = Step(args.n, args.precision, device)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=device)   # > L2 (129 MB)

    def barrier():
        if world > 1:
            dist.barrier()

    for _ in range(args.warmup):
        step.run()
    torch.cuda.synchronize()

    # FP32 peak on this device, measured (denominator of the roofline)
    sink = torch.zeros(1, dtype=torch.float32, device=device)
    iters = 1 << 16
    _capi.check(lib.fvx_probe_fp32_fma(8, 16, sink.data_ptr(), None))
    torch.cuda.synchronize()
    ps, pe = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ps.record()
    _capi.check(lib.fvx_probe_fp32_fma(8, iters, sink.data_ptr(), None))
    pe.record()
    torch.cuda.synchronize()
    sms = torch.cuda.get_device_properties(device).multi_processor_count
    fp32_peak = 8 * sms * 256 * iters * 16 / (ps.elapsed_time(pe) * 1e-3)

    clocks = start_clock_sampler()
    step.field.sweep_events = []
    launches0 = lib.fvx_launch_count()
    step_ms = []
    for _ in range(args.steps):
        flush.zero_()
        barrier()
        torch.cuda.synchronize()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        step.run()
        e.record()
        torch.cuda.synchronize()
        barrier()
        step_ms.append(s.elapsed_time(e))
    launches = lib.fvx_launch_count() - launches0
    clk = stop_clock_sampler(clocks, local)
    events = step.field.sweep_events
    step.field.sweep_events = None
    ms = sum(step_ms) / len(step_ms)
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    ms_max = float(t.item())
    value = world * 1e3 / ms_max

    # per-kind sweep durations inside the timed steps
    kinds = {}
    for mode, kern, nt, ns, a, b in events:
        key = (MODE_NAMES[mode], kern, nt, ns)
        kinds.setdefault(key, []).append(a.elapsed_time(b))
    dom = max(kinds.items(), key=lambda kv: sum(kv[1]))
    (mname, kern, nt, ns), durs = dom
    avg_ms = sum(durs) / len(durs)
    flop = FLOP_PER_PAIR.get((mname, kern), 0) * nt * ns
    achieved = flop / (avg_ms * 1e-3) / 1e12

    result = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_max,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32c sweeps / f64 integration" if args.precision == "f32c" else "f64",
        "data": "synthetic (seeded slab wake, BASELINE config-3 shapes)",
        "config": {"workload": f"slab wake, {args.n} particles + 4096 collocation points, "
                               "one RK3 free-wake step with stretching and relaxation",
                   "particles": args.n, "collocation_points": 4096,
                   "precision": args.precision, "kernel": "winckelmans",
                   "relax_kernel": "gaussianerf", "l2": "flushed (256 MB write) before each step",
                   "parallelism": f"replicas x{world}"},
        "gpu_launches": int(launches),
        "clocks": clk,
        "roofline": {"bound": "fp32", "kernel": f"pairs_kernel<{mname},{kern}>",
                     "achieved": achieved, "peak": fp32_peak / 1e12, "unit": "TFLOP/s",
                     "frac": achieved / (fp32_peak / 1e12), "traffic": None,
                     "flop_per_launch": flop, "avg_launch_ms": avg_ms,
                     "peak_source": "measured FP32 FMA probe (fvx_probe_fp32_fma) on this GPU"},
        "sweep_ms": {f"{k[0]}/{k[1]}/{k[2]}x{k[3]}": sum(v) / len(v) for k, v in kinds.items()},
    }

    if not args.no_baselines and rank == 0:
        n_t = 4096
        f64_s = sample_sweeps(step.field, n_t, "f64")
        f32_s = sample_sweeps(step.field, n_t, args.precision)
        result["fp64_direct"] = {"step_s_extrapolated": f64_s, "steps_per_s": 1.0 / f64_s,
                                 "sample": f"{n_t} targets x {args.n} sources per sweep kind",
                                 "same_sample_f32c_step_s": f32_s,
                                 "speedup_vs_fp64": f64_s * 1e3 / ms_max}
        # wake-on-collocation accuracy of the mixed form against FP64
        u32 = step.u_colloc.clone()
        step.field.precision = "f64"
        u64 = torch.empty_like(u32)
        step.field._sweep(0, step.colloc, None, step.colloc.shape[0], u64)
        step.field.precision = args.precision
        step.field._sweep(0, step.colloc, None, step.colloc.shape[0], u32)
        torch.cuda.synchronize()
        err = float((u32 - u64).abs().max() / u64.abs().max())
        result["fp64_direct"]["colloc_velocity_rel_err"] = err
        cores = os.cpu_count() or 1
        cpu_s, thr, detail = cpu_oracle_step_seconds(step.host, 64, cores)
        result["cpu_baseline"] = {"value": 1.0 / cpu_s, "unit": UNIT, "cores": thr,
                                  "kind": "port",
                                  "sample": f"{detail['targets']} targets x {detail['sources']} "
                                            "sources per sweep kind, FP64 C oracle with OpenMP, "
                                            "scaled to the full step by N/targets"}

    if not args.no_e2e:
        # End to end through the host-facing API: pinned host state in, step,
        # new state + collocation velocities out, every step.
        f = step.field
        n = f.np
        hp = torch.empty((n, 3), dtype=torch.float64).pin_memory()
        hg = torch.empty((n, 3), dtype=torch.float64).pin_memory()
        hs = torch.empty(n, dtype=torch.float64).pin_memory()
        hu = torch.empty((4096, 3), dtype=torch.float64).pin_memory()
        hp.copy_(f._pos[:n])
        hg.copy_(f._gamma[:n])
        hs.copy_(f._sigma[:n])
        torch.cuda.synchronize()
        e2e_steps = 1
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        barrier()
        s.record()
        for _ in range(e2e_steps):
            f._pos[:n].copy_(hp, non_blocking=True)
            f._gamma[:n].copy_(hg, non_blocking=True)
            f._sigma[:n].copy_(hs, non_blocking=True)
            step.run()
            hp.copy_(f._pos[:n], non_blocking=True)
            hg.copy_(f._gamma[:n], non_blocking=True)
            hs.copy_(f._sigma[:n], non_blocking=True)
            hu.copy_(step.u_colloc, non_blocking=True)
        e.record()
        torch.cuda.synchronize()
        e2e_ms = s.elapsed_time(e) / e2e_steps
        t = torch.tensor([e2e_ms], dtype=torch.float64, device=device)
        if world > 1:
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
        h2d = n * (3 + 3 + 1) * 8
        d2h = n * (3 + 3 + 1) * 8 + 4096 * 3 * 8
        result["e2e"] = {"value": world * 1e3 / float(t.item()), "unit": UNIT,
                         "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h}

    if rank == 0:
        print(json.dumps(result))


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        backend = "gloo" if args.impl == "reference" else "nccl"
        dist.init_process_group(backend)
    try:
        if args.impl == "reference":
            run_reference(args, rank, world)
        else:
            run_ours(args, rank, world)
    finally:
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
