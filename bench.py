#!/usr/bin/env python
"""Benchmark of the VPM+panel step (hybrid panel-particle induction) on one GB300.

Workload (``Step``): the large flapping configuration (NACA 2412 main wing
in two halves + NACA 0012 V-tail, 3 surfaces, 192 panels, N_keep = 10 ring
rows; ``geometry.flapping_aircraft``) with its particle wake seeded to 2^20
(~1e6) particles by a seeded 20c x 10c x 2c slab behind the tail
(``fluxvortex_gb300.workloads.slab_wake``).  One step = lattice + AIC +
wake-on-collocation (ring rows + every particle) + FP64 LU solve + loads
(CL, CDi) + shedding + row-to-particle conversion + one RK3 particle step
with free wake and stretching (3 velocity + 3 stretching all-pairs sweeps),
all resident in HBM.  Sweeps run FP32 with compensated accumulation
(``--precision f32c``) or FP64; panel side and time integration are FP64.

Output: one JSON line (rank 0).  ``value`` = steps/s of the whole job
(device-timed, inputs resident, L2 flushed before every step); ``e2e`` = the
same through the host-facing API (particle state copied in from pinned host
memory, new state and CL/CDi copied back, every step); ``fp64_direct`` = the
same step with FP64 sweeps, timed on a target sample and scaled (all-pairs
cost is linear in the target count), plus the CL/CDi error of the mixed form
against FP64 sweeps at the same state; ``cpu_baseline`` = the FP64 C oracle
on the host cores on a bounded target sample, scaled likewise.

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
# sqrt / rsqrt / div / exp / erf as 1, with the per-source constants (sigma^2,
# 2.5 sigma^2, the 1/4pi folded into the strengths) hoisted out of the pair.
FLOP_PER_PAIR = {
    ("velocity", "winckelmans"): 30,
    ("stretch", "winckelmans"): 57,
    ("vorticity", "winckelmans"): 45,
    ("vorticity", "gaussianerf"): 55,
    ("velocity", "gaussianerf"): 40,
    ("stretch", "gaussianerf"): 67,
}
WORKLOAD = ("VPM+panel step: flapping NACA2412 wing + NACA0012 V-tail, 3 surfaces, 192 panels "
            "+ {n} seeded wake particles (cores 1.3 x spacing), RK3 free wake with stretching "
            "on, Pedrizzetti relaxation off, converted cores 1.3 x mean ring edge")
# Algorithmic flop of one far-field (target particle, cell) evaluation of the
# treecode's quadrupole expansion (same counting convention).
M2P_FLOP = {"velocity": 166, "stretch": 355, "vorticity": 300}
# ... and of one local-expansion application per target particle (L2P)
L2P_FLOP = {"velocity": 90, "stretch": 80, "vorticity": 60}
# tensor flop of the far-field network per (leaf, cell) pair: 2 x MACs of the
# 48-128-128-128-32 layers
MLP_FLOP_PER_PAIR = 2 * (48 * 128 + 128 * 128 + 128 * 128 + 128 * 32)
# dram__bytes_read.sum + dram__bytes_write.sum of one launch of the stretching
# evaluation kernel on the 2^20-particle slab at this leaf target, from the ncu
# capture summarised in ``source`` (which gives the command and the commit)
EVAL_TRAFFIC = {"bytes": 1.5079e8, "leaf": 32,
                "source": "profiles/eval_kernel_phased_tiles_slab_1e6_leaf32.md"}
MODE_NAMES = {0: "velocity", 1: "stretch", 2: "velocity_stretch", 3: "jacobian", 4: "vorticity"}


def _bf16_peak():
    """Dense BF16 tensor peak: measured (MEASURED_PEAKS.json) or the fallback."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            pk = json.load(f)
        for k in ("bf16_tflops", "bf16_dense_tflops"):
            if k in pk and pk[k]:
                return float(pk[k]), "measured (MEASURED_PEAKS.json " + k + ")"
    except (OSError, ValueError):
        pass
    return 1900.0, "fallback 1.9 PFLOP/s (no measured peak file)"


BF16_PEAK_TFLOPS, BF16_PEAK_SOURCE = _bf16_peak()


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--particles", "--n", dest="n", type=int, default=1 << 20,
                   help="particles (spell it --particles under torchrun, whose own options "
                        "share the --n prefix)")
    p.add_argument("--precision", default="f32c", choices=["f32c", "f64"])
    p.add_argument("--far-field", default="learned",
                   choices=["direct", "tree", "m2p", "m2l", "learned"],
                   help="particle self-sweeps: direct all-pairs, or the treecode with the "
                        "accepted cells per target particle (tree = m2p), as analytic local "
                        "expansions (m2l), or through the learned far-field operator")
    p.add_argument("--leaf", type=int, default=32, help="treecode particles per leaf")
    p.add_argument("--no-flutter", dest="flutter", action="store_false",
                   help="skip the batched flutter-sweep measurement")
    p.add_argument("--cl-steps", type=int, default=43,
                   help="steps of the CL-history check against direct sweeps (0: off; 43 = "
                        "one flapping cycle)")
    p.add_argument("--cl-particles", type=int, default=1 << 18,
                   help="seeded particles of the CL-history check")
    p.add_argument("--e2e-steps", type=int, default=5,
                   help="steps of the end-to-end measurement (0: off)")
    p.add_argument("--relax-steps", type=int, default=3,
                   help="timed steps of each variant of the step: with the Pedrizzetti "
                        "relaxation, and without the stretching term (0: off)")
    p.add_argument("--no-baselines", action="store_true")
    p.add_argument("--sweep-case", action="store_true",
                   help="instead of the step: one treecode velocity + stretching sweep pair of "
                        "the seeded slab (the profiling case of the evaluation and network "
                        "kernels); --repeat R more pairs print median kernel times")
    p.add_argument("--repeat", type=int, default=0)
    p.add_argument("--sweep-core", choices=("thin", "resolved"), default="thin",
                   help="--sweep-case cores: 0.02c (the slab sweep case) or 1.3 x the "
                        "particle spacing (the benchmarked step's slab)")
    p.add_argument("--sweep-kind", choices=("velocity-stretch", "vorticity"),
                   default="velocity-stretch",
                   help="--sweep-case sweeps: the Winckelmans velocity + stretching pair, or "
                        "the Gaussian-erf vorticity sweep of the Pedrizzetti relaxation")
    return p.parse_args()


_T0 = time.perf_counter()


def progress(msg):
    """One line per bench phase on stderr (stdout carries only the JSON line)."""
    print(f"[bench {time.perf_counter() - _T0:8.1f}s] {msg}", file=sys.stderr, flush=True)


# ---------------------------------------------------------------------------
CLOCK_QUERY = ("uuid,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
               "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
               "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")


def device_uuid(device):
    """nvidia-smi's identifier ("GPU-<uuid>") of a CUDA device.  nvidia-smi
    numbers GPUs in PCI order, whatever CUDA_VISIBLE_DEVICES says, so the
    process-local CUDA ordinal cannot select the GPU's rows; its UUID can."""
    import torch
    u = getattr(torch.cuda.get_device_properties(device), "uuid", None)
    if u is None:
        return None
    s = str(u)
    return s if s.startswith("GPU-") else "GPU-" + s


def parse_clock_samples(lines, gpu_uuid):
    """Summary of nvidia-smi rows (``CLOCK_QUERY`` order, csv, no header, no
    units) of the GPU whose UUID is ``gpu_uuid``: median SM clock under load,
    the maximum clock, and every throttle reason seen active."""
    sm, smax, reasons = [], [], set()
    names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
    want = (gpu_uuid or "").lower()
    for line in lines:
        parts = [x.strip() for x in line.split(",")]
        if len(parts) < 10 or parts[0].lower() != want:
            continue
        try:
            sm.append(float(parts[2]))
            smax.append(float(parts[3]))
        except ValueError:
            continue
        for nm, v in zip(names, parts[6:10]):
            if v.lower() == "active":
                reasons.add(nm)
    if not sm:
        return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
    loaded = [x for x in sm if x > 0.5 * max(sm)] or sm
    return {"sm_mhz": statistics.median(loaded), "sm_max_mhz": max(smax),
            "reasons": sorted(reasons), "samples": len(sm), "gpu": gpu_uuid}


def start_clock_sampler():
    path = tempfile.mktemp(prefix="clocks_", suffix=".csv")
    q = CLOCK_QUERY
    try:
        f = open(path, "w")
        proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                 "-lms", "50"], stdout=f, stderr=subprocess.DEVNULL)
        # the timed steps start once the sampler has written its first line
        # (nvidia-smi takes a few hundred ms to start)
        t_end = time.perf_counter() + 3.0
        while time.perf_counter() < t_end and os.path.getsize(path) == 0 and proc.poll() is None:
            time.sleep(0.02)
        return proc, f, path
    except (OSError, FileNotFoundError):
        return None, None, path


def stop_clock_sampler(handle, gpu_uuid):
    proc, f, path = handle
    if proc is None:
        return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
    proc.terminate()
    try:
        proc.wait(timeout=5)
    except subprocess.TimeoutExpired:
        proc.kill()
    f.close()
    with open(path) as fh:
        out = parse_clock_samples(fh.readlines(), gpu_uuid)
    os.unlink(path)
    return out


# ---------------------------------------------------------------------------
class Step:
    """The benchmarked VPM+panel step on one device (state resident in HBM).

    Geometry: the large flapping configuration (main wing NACA 2412, root /
    tip chord 1.75 / 1.5, semi-span 6, two halves of nc=6 x ns=8 cosine; V-tail
    NACA 0012, chord 1.5 / 1.0, semi-span 2, 6 x 16; 3 surfaces, 192 panels;
    15 deg flapping, period 1 s, V=10 m/s, alpha=1 deg, 43 steps per cycle,
    N_keep=10 ring rows).  Its particle wake is seeded with the slab wake of
    ``workloads.slab_wake(n)`` (2^20 particles behind the tail) and grows by
    one converted ring row (32 strips x 4 = 128 particles) per step.  A step: lattice,
    AIC, wake-on-collocation (rings + all particles), FP64 LU solve, loads
    (CL, CDi), shedding, conversion, and one RK3 particle step with free wake
    and stretching (3 velocity + 3 stretching sweeps over all particles)."""

    def __init__(self, n, precision, device, steps_hint=64, far_field="direct", leaf=64,
                 rlxf=0.0, stretch=True):
        import torch
        from fluxvortex_gb300.geometry import flapping_aircraft
        from fluxvortex_gb300.hybrid import HybridStep
        from fluxvortex_gb300.workloads import AIRCRAFT_SLAB_X0, resolved_core, slab_wake
        # the seeded slab stands in for the grown wake: cores of 1.3 x the
        # particle spacing, like the converted particles' (resolved_core)
        pos, gam, sig, colloc = slab_wake(n, x0=AIRCRAFT_SLAB_X0, sigma=resolved_core(n))
        self.host = dict(pos=pos, gamma=gam, sigma=sig, colloc=colloc)
        # converted particles take the core 1.3 x the ring's mean edge, the
        # hybrid configurations' rule (the core |V| dt sits below the particle
        # spacing, and the converted wake is then chaotic: a 1e-12 change of
        # the state reaches the CL history within a cycle)
        self.cfg = flapping_aircraft(n_keep=10, free_vpm=True, stretch=stretch, rlxf=rlxf,
                                     sigma_rule="edge",
                                     max_particles=n + 128 * (steps_hint + 8),
                                     far_field=None if far_field == "direct" else far_field)
        self.hs = HybridStep(self.cfg, precision=precision, device=device)
        if self.hs.field.tree is not None:
            self.hs.field.tree.leaf_target = leaf
        self.hs.field.add_particles_batch(pos, gam, sig)
        self.field = self.hs.field
        self.device = device

    def run(self):
        self.hs.step()

def sample_sweeps(field, n_t, precision, reps=1, panels=192):
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
             "stretch": (_capi.PAIR_STRETCH, tg, "winckelmans")}
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
    # 3 velocity + 3 stretching sweeps over all N targets, plus the
    # collocation and bound-leg sweeps (2 x panels targets)
    return (3 * sec["velocity"] + 3 * sec["stretch"]) * full + sec["velocity"] * 2 * panels / n_t


def cpu_oracle_step_seconds(host, n_t, threads=None, panels=192):
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
    scale = n / n_t
    # step: 3 velocity + 3 stretching sweeps (a velocity+stretching pass bounds
    # the stretching pass) + collocation and bound-leg sweeps (2 x panels)
    step = (3 * t_vel + 3 * t_vs) * scale + t_vel * 2 * panels / n_t
    return step, O.num_threads(), dict(velocity_s=t_vel, stretch_s=t_vs,
                                       targets=n_t, sources=n)


# ---------------------------------------------------------------------------
def flutter_sweep_measure(args):
    """The batched flutter sweep (Goland wing, 64 airspeeds over 80-180 m/s,
    100 chords of travel each: 339..762 steps, particle wakes of uneven
    length): one persistent launch per sweep replayed from a CUDA graph, with
    the aerodynamic particle sums in FP32 (compensated) and in FP64; flutter
    speeds of both, and the FP64 CPU oracle's time for one environment step
    scaled to the sweep."""
    import numpy as np
    import torch
    from fluxvortex_gb300.flutter import FlutterSweep, goland
    cfg = goland()
    V = cfg.velocities(64)
    out = {"workload": "Goland wing 8x4 panels, beam 8 elements, 64 airspeeds 80-180 m/s, "
                       f"{cfg.num_chords:g} chords, n_keep {cfg.n_keep}, "
                       f"<= {cfg.max_particles} particles per environment",
           "steps_per_env": [int(min(cfg.n_steps(v) for v in V)), int(max(cfg.n_steps(v) for v in V))]}
    for prec in ("f32c", "f64"):
        sw = FlutterSweep(cfg, V, precision=prec, threads="auto")
        sw.run(graph=True)                    # capture + first replay
        torch.cuda.synchronize()
        ms = []
        for _ in range(3):
            sw.reset()
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record()
            sw.run(graph=True)
            e.record()
            torch.cuda.synchronize()
            ms.append(s.elapsed_time(e))
        total_steps = int(sw.steps.sum())
        out[prec] = {"sweep_ms": min(ms), "env_steps_per_s": total_steps / (min(ms) * 1e-3),
                     "threads_per_env": sw.threads, "flutter_speed_mps": sw.flutter_speed()}
    a, b = out["f32c"]["flutter_speed_mps"], out["f64"]["flutter_speed_mps"]
    out["flutter_speed_diff_mps"] = None if a is None or b is None else abs(a - b)
    if not args.no_baselines:
        import time as _t
        from oracle.flutter import FlutterOracle
        o = FlutterOracle(cfg, float(V[0]))
        for _ in range(30):                   # wake rows start converting after n_keep
            o.step()
        t0 = _t.perf_counter()
        for _ in range(10):
            o.step()
        per_step = (_t.perf_counter() - t0) / 10
        out["cpu_oracle"] = {"s_per_env_step": per_step,
                             "sweep_s_extrapolated": per_step * int(sw.steps.sum()),
                             "kind": "port", "cores": 1,
                             "sample": "10 steps of the 80 m/s environment after 30 warm-up steps"}
    return out


def run_sweep_case(args):
    """One treecode self-sweep pair (velocity, then stretching) of the seeded
    slab wake (``workloads.slab_wake``: uniform in a 20c x 10c x 2c slab,
    sigma 0.02c, or with ``--sweep-core resolved`` 1.3 x the particle spacing
    as in the benchmarked step) with the chosen far field and FP64 validation
    off: the
    smallest complete invocation of the particle hot path, used as the
    profiling case of the evaluation, translation and network kernels.
    ``--repeat R`` runs R more sweep pairs at the same positions and prints the
    median times of the evaluation kernel and of the local-expansion stage
    (CUDA events inside the library).  ``--sweep-kind vorticity`` runs the
    Gaussian-erf vorticity sweep of the relaxation instead of the pair."""
    import torch
    from fluxvortex_gb300 import _capi
    from fluxvortex_gb300.tree import TreeSweeper
    from fluxvortex_gb300.workloads import resolved_core, slab_wake
    ff = {"tree": "m2p", "direct": "m2p"}.get(args.far_field, args.far_field)
    core = resolved_core(args.n) if args.sweep_core == "resolved" else None
    pos, gam, sig, _ = slab_wake(args.n, sigma=core)
    d = lambda x: torch.as_tensor(x, dtype=torch.float64, device="cuda")  # noqa: E731
    P, G, S = d(pos), d(gam), d(sig)
    ts = TreeSweeper(theta=0.5, leaf_target=args.leaf)
    mlp = None
    if ff == "learned":
        from fluxvortex_gb300.learned import FarFieldMLP
        mlp = FarFieldMLP.load()
    ts.set_far_field(ff, mlp=mlp)
    ts.set_validation(0, 0.1)
    out = torch.empty((args.n, 3), dtype=torch.float64, device="cuda")
    if args.sweep_kind == "vorticity":
        kinds = (("vorticity", _capi.PAIR_VORTICITY, None, "gaussianerf"),)
    else:
        kinds = (("velocity", _capi.PAIR_VELOCITY, None, "winckelmans"),
                 ("stretch", _capi.PAIR_STRETCH, G, "winckelmans"))
    for _, mode, tg, kern in kinds:
        ts.sweep(mode, kern, P, G, S, args.n, out, tgt_gamma=tg)
    times = {k[0]: [] for k in kinds}
    for _ in range(args.repeat):
        for name, mode, tg, kern in kinds:
            ts.sweep(mode, kern, P, G, S, args.n, out, tgt_gamma=tg, check=True,
                     same_positions=True)
            loc = ts.last_local_ms() if ff != "m2p" else 0.0
            times[name].append((ts.last_eval_ms(), loc))
    torch.cuda.synchronize()
    for name, t in times.items():
        if t:
            ev = sorted(x[0] for x in t)[len(t) // 2]
            lo = sorted(x[1] for x in t)[len(t) // 2]
            print(f"{name}: evaluation {ev:.3f} ms, local-expansion stage {lo:.3f} ms "
                  f"(median of {len(t)})", file=sys.stderr)
    st = _capi.status_read_and_clear()
    print(f"sweep case ok: max |out| = {float(out.abs().max())}, status {st}", file=sys.stderr)
    if st:
        raise SystemExit(f"device status {st}")


def max_over_ranks(value, world, device=None):
    """The largest of every rank's value (the job's time is its slowest rank's)."""
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    if world > 1:
        import torch.distributed as dist
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_reference(args, rank, world):
    if rank != 0:
        return
    from fluxvortex_gb300.workloads import AIRCRAFT_SLAB_X0, resolved_core, slab_wake
    pos, gam, sig, colloc = slab_wake(args.n, x0=AIRCRAFT_SLAB_X0, sigma=resolved_core(args.n))
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
    sample = (f"{n_t} targets x {args.n} sources per sweep kind (velocity, velocity+stretching),"
              f" scaled to the full step by N/targets")
    # the reference's own NumPy particle path (kernel.py, one thread), restated
    # with its block structure, at 2^14 and 2^16 particles on 512 targets,
    # scaled by N/targets and then to the benchmarked N by (N / n)^2
    from oracle import numpy_reference as NR
    numpy_ref = {"kind": "port of the reference's NumPy kernels (kernel.py:69-190), "
                         "blocks of 512, FP64", "cores": 1, "sizes": {}}
    for n_np in (1 << 14, 1 << 16):
        p, g, sgm, _ = slab_wake(n_np, x0=AIRCRAFT_SLAB_X0, sigma=resolved_core(n_np))
        s_np, det = NR.step_seconds(p, g, sgm, min(512, n_np))
        numpy_ref["sizes"][str(n_np)] = {
            "step_s": s_np, **det,
            "step_s_extrapolated_to_n": s_np * (args.n / n_np) ** 2,
            "extrapolation": f"N^2 from {n_np} to {args.n} particles (extrapolated, not run)"}
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_s * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": WORKLOAD.format(n=args.n)},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": thr, "kind": "port",
                         "sample": sample},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "numpy_reference": numpy_ref,
    }))


def run_ours(args, rank, world):
    import torch
    import torch.distributed as dist
    from fluxvortex_gb300 import _capi

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    device = torch.device("cuda", local)
    lib = _capi.load()

    progress(f"building the step: {args.n} particles, far field {args.far_field}")
    step = Step(args.n, args.precision, device, far_field=args.far_field, leaf=args.leaf)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=device)   # > L2 (129 MB)
    progress("warm-up")

    def barrier():
        if world > 1:
            dist.barrier()

    for _ in range(args.warmup):
        step.run()
    torch.cuda.synchronize()
    # every timed step starts from this state: the seeded slab (cores 0.02c,
    # below the 0.074c particle spacing) is an under-resolved random vorticity
    # field that the reference's stretching and core-size update drive to the
    # strength and core clamps within about ten steps, and the tree's work
    # would drift with it
    snap = step.hs.snapshot()

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

    progress("timed steps")
    clocks = start_clock_sampler()
    step.field.sweep_events = []
    launches0 = lib.fvx_launch_count()
    step_ms = []
    for _ in range(args.steps):
        step.hs.restore(snap)
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
    clk = stop_clock_sampler(clocks, device_uuid(device))
    events = step.field.sweep_events
    step.field.sweep_events = None
    ms = sum(step_ms) / len(step_ms)
    ms_max = max_over_ranks(ms, world, device)
    value = world * 1e3 / ms_max

    # per-kind sweep durations inside the timed steps
    kinds = {}
    for mode, kern, nt, ns, a, b in events:
        key = (MODE_NAMES[mode], kern, nt, ns)
        kinds.setdefault(key, []).append(a.elapsed_time(b))
    # the dominant kernel: for treecode sweeps the evaluation kernel with the
    # most launch time (its own CUDA events), else the sweep kind with the most
    dom = max(kinds.items(), key=lambda kv: sum(kv[1]))
    tree_kinds = [kv for kv in kinds.items() if kv[0][1].startswith("tree/")]
    if tree_kinds and step.field.tree_events:
        def _eval_total(kv):
            m = kv[0][0]
            return sum(e[3] for e in step.field.tree_events if MODE_NAMES[e[0]] == m)
        dom = max(tree_kinds, key=_eval_total)
    (mname, kern, nt, ns), durs = dom
    avg_ms = sum(durs) / len(durs)
    flop = FLOP_PER_PAIR.get((mname, kern), 0) * nt * ns
    kname = f"pairs_kernel<{mname},{kern}>"
    if kern.startswith("tree/"):
        # treecode: the evaluation kernel's algorithmic work is its near pairs
        # plus its far (target, cell) expansions; its own launch time is timed
        # with CUDA events around the launch inside the library
        tev = [e for e in step.field.tree_events if MODE_NAMES[e[0]] == mname]
        base = kern.split("/", 1)[1]
        has_local_exp = step.field.far_field in ("m2l", "learned")
        flop = sum(FLOP_PER_PAIR[(mname, base)] * e[2][6] + M2P_FLOP[mname] * e[2][7]
                   + (L2P_FLOP[mname] * args.n if has_local_exp else 0) for e in tev) / len(tev)
        avg_ms = sum(e[3] for e in tev) / len(tev)
        kname = f"tree eval_kernel<{mname},{base}>"
        tree_stats = {"levels": int(tev[-1][2][0]), "leaves": int(tev[-1][2][1]),
                      "near_pairs": int(tev[-1][2][6]), "far_target_cell_pairs": int(tev[-1][2][7]),
                      "local_expansion_pairs": int(tev[-1][2][4]),
                      "eval_ms": avg_ms,
                      "local_ms": sum(e[4] for e in tev) / len(tev),
                      "sweep_ms": sum(durs) / len(durs)}
        vals = [e[5] for e in step.field.tree_events if e[5]]
        if vals:
            tree_stats["validation_per_step"] = vals[-1]
    achieved = flop / (avg_ms * 1e-3) / 1e12
    # DRAM bytes per launch of the stretching evaluation from one ncu capture
    # of the same kernel on the same workload (EVAL_TRAFFIC names the capture's
    # summary); reported only for the workload that capture matches
    traffic, traffic_source = None, None
    if (kname == "tree eval_kernel<stretch,winckelmans>" and args.n == 1 << 20
            and args.leaf == EVAL_TRAFFIC["leaf"] and args.precision == "f32c"):
        traffic, traffic_source = EVAL_TRAFFIC["bytes"], EVAL_TRAFFIC["source"]

    result = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_max,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32c sweeps / f64 integration" if args.precision == "f32c" else "f64",
        "data": "synthetic (flapping-aircraft geometry; wake seeded with a 20c x 10c x 2c slab of particles behind the tail)",
        "config": {"workload": WORKLOAD.format(n=args.n), "particles": args.n,
                   "panels": step.hs.P, "n_keep": step.cfg.n_keep,
                   "precision": args.precision, "kernel": "winckelmans",
                   "l2": "flushed (256 MB write) before each step",
                   "state": f"each timed step restarts from the state after {args.warmup} "
                            "warm-up steps (restored outside the timed region)",
                   "parallelism": f"replicas x{world}"},
        "gpu_launches": int(launches),
        "clocks": clk,
        "roofline": {"bound": "fp32", "kernel": kname,
                     "achieved": achieved, "peak": fp32_peak / 1e12, "unit": "TFLOP/s",
                     "frac": achieved / (fp32_peak / 1e12), "traffic": traffic,
                     "traffic_unit": "bytes per launch (ncu capture)",
                     "traffic_source": traffic_source,
                     "flop_per_launch": flop, "avg_launch_ms": avg_ms,
                     "peak_source": "measured FP32 FMA probe (fvx_probe_fp32_fma) on this GPU"},
        "sweep_ms": {f"{k[0]}/{k[1]}/{k[2]}x{k[3]}": sum(v) / len(v) for k, v in kinds.items()},
    }
    if kern.startswith("tree/"):
        result["config"]["far_field"] = {"method": f"treecode/{step.field.far_field}",
                                         "theta": step.field.tree.theta,
                                         "leaf_target": step.field.tree.leaf_target, **tree_stats}
        if step.field.far_field == "learned" and tree_stats["local_ms"] > 0:
            # the network stage (features, analytic translation, four tcgen05
            # layers, accumulation) against the tensor peak
            mlp_tf = (MLP_FLOP_PER_PAIR * tree_stats["local_expansion_pairs"]
                      / (tree_stats["local_ms"] * 1e-3) / 1e12)
            result["roofline_mlp"] = {
                "bound": "tensor", "kernel": "farfield_kernel + m2l_pairs_kernel (local stage)",
                "achieved": mlp_tf,
                "peak": BF16_PEAK_TFLOPS, "unit": "TFLOP/s", "frac": mlp_tf / BF16_PEAK_TFLOPS,
                "peak_source": BF16_PEAK_SOURCE}

    if not args.no_baselines and rank == 0:
        # FP64 direct form of the same step: every sweep in FP64 on a target
        # sample large enough to fill the GPU, scaled by N / targets (all-pairs
        # work is linear in the target count)
        n_t = 32768
        progress("FP64 direct sample")
        f64_s = sample_sweeps(step.field, n_t, "f64")
        result["fp64_direct"] = {"step_s_extrapolated": f64_s,
                                 "steps_per_s": 1.0 / f64_s,
                                 "sample": f"{n_t} targets x {args.n} sources per sweep kind, "
                                           "scaled by N/targets",
                                 "speedup_vs_fp64": f64_s * 1e3 / ms_max}
        # CL / CDi of the mixed form against FP64 particle sweeps, same state
        cl64, cdi64 = step.hs.panel_loads("f64")
        cl32, cdi32 = step.hs.panel_loads(args.precision)
        result["fp64_direct"]["cl_rel_err_same_state"] = abs(cl32 - cl64) / abs(cl64)
        result["fp64_direct"]["cdi_rel_err_same_state"] = abs(cdi32 - cdi64) / abs(cdi64)
        result["fp64_direct"]["cl"] = cl64
        cores = os.cpu_count() or 1
        progress("CPU baseline")
        cpu_s, thr, detail = cpu_oracle_step_seconds(step.host, 64, cores)
        result["cpu_baseline"] = {"value": 1.0 / cpu_s, "unit": UNIT, "cores": thr,
                                  "kind": "port",
                                  "sample": f"{detail['targets']} targets x {detail['sources']} "
                                            "sources per sweep kind, FP64 C oracle with OpenMP, "
                                            "scaled to the full step by N/targets"}

    if args.flutter and rank == 0:
        progress("flutter sweep")
        result["flutter_sweep"] = flutter_sweep_measure(args)

    if args.e2e_steps > 0:
        # End to end through the host-facing API, every step: the particle
        # state (positions, strengths, cores) in from pinned host memory, the
        # step, the new state and CL / CDi back out; the host holds the state
        # between steps, so each step continues from the last one's output.
        progress("end to end")
        step.hs.restore(snap)
        f = step.field
        n0 = f.np
        cap = n0 + 128 * (args.e2e_steps + 1)
        hp = torch.empty((cap, 3), dtype=torch.float64).pin_memory()
        hg = torch.empty((cap, 3), dtype=torch.float64).pin_memory()
        hs = torch.empty(cap, dtype=torch.float64).pin_memory()
        hc = torch.empty((args.e2e_steps, 2), dtype=torch.float64).pin_memory()
        hp[:n0].copy_(f._pos[:n0])
        hg[:n0].copy_(f._gamma[:n0])
        hs[:n0].copy_(f._sigma[:n0])
        torch.cuda.synchronize()
        h2d = d2h = 0
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        barrier()
        s.record()
        for k in range(args.e2e_steps):
            n = f.np
            f._pos[:n].copy_(hp[:n], non_blocking=True)
            f._gamma[:n].copy_(hg[:n], non_blocking=True)
            f._sigma[:n].copy_(hs[:n], non_blocking=True)
            h2d += n * 7 * 8
            f.positions_changed()
            step.run()
            m = f.np
            kk = step.hs.k - 1
            hp[:m].copy_(f._pos[:m], non_blocking=True)
            hg[:m].copy_(f._gamma[:m], non_blocking=True)
            hs[:m].copy_(f._sigma[:m], non_blocking=True)
            hc[k, 0:1].copy_(step.hs._cl[kk:kk + 1], non_blocking=True)
            hc[k, 1:2].copy_(step.hs._cdi[kk:kk + 1], non_blocking=True)
            d2h += m * 7 * 8 + 16
        e.record()
        torch.cuda.synchronize()
        e2e_ms = max_over_ranks(s.elapsed_time(e) / args.e2e_steps, world, device)
        result["e2e"] = {"value": world * 1e3 / e2e_ms, "unit": UNIT,
                         "h2d_bytes_per_step": h2d // args.e2e_steps,
                         "d2h_bytes_per_step": d2h // args.e2e_steps,
                         "steps": args.e2e_steps, "ms_per_step": e2e_ms}

    if args.relax_steps > 0 and rank == 0:
        # the same step in other forms, timed alike: with the reference's
        # Pedrizzetti relaxation (rlxf = 0.3: one Gaussian-erf vorticity
        # self-sweep and the strength update more); as the reference's hybrid
        # solver runs its free wake, without the stretching term
        # (experiment_hybrid_panel_particle.py:140-143: three velocity sweeps);
        # both, as that solver is set up (rlxf = 0.3 at :111); and with the
        # analytic translation alone as the far field
        del step
        torch.cuda.empty_cache()
        flush = torch.empty(256 << 20, dtype=torch.uint8, device=device)
        for key, kw, note in (
                ("relaxation_variant", dict(rlxf=0.3),
                 "the benchmarked step plus the reference's Pedrizzetti relaxation (a "
                 "Gaussian-erf vorticity self-sweep and the strength update)"),
                ("stretching_off_variant", dict(stretch=False),
                 "the benchmarked step without the stretching term, as the reference's "
                 "hybrid solver runs its free wake (3 velocity self-sweeps per step)"),
                ("reference_solver_variant", dict(stretch=False, rlxf=0.3),
                 "the step as the reference's hybrid solver sets it up: no stretching "
                 "term, Pedrizzetti relaxation at rlxf = 0.3 (3 velocity self-sweeps and "
                 "one Gaussian-erf vorticity self-sweep per step)"),
                ("translation_only_variant", dict(far_field="m2l"),
                 "the benchmarked step with the analytic multipole-to-local translation "
                 "alone as the far field (no network residual), judged alike: the method "
                 "without the learned part")):
            progress(key)
            st3 = Step(args.n, args.precision, device, leaf=args.leaf,
                       **{"far_field": args.far_field, **kw})
            for _ in range(args.warmup):
                st3.run()
            snap3 = st3.hs.snapshot()
            ms3 = []
            for _ in range(args.relax_steps):
                st3.hs.restore(snap3)
                flush.zero_()
                torch.cuda.synchronize()
                s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                s.record()
                st3.run()
                e.record()
                torch.cuda.synchronize()
                ms3.append(s.elapsed_time(e))
            result[key] = {**kw, "ms_per_step": sum(ms3) / len(ms3),
                           "steps_per_s": 1e3 * len(ms3) / sum(ms3), "steps": len(ms3),
                           "note": note}
            del st3
            torch.cuda.empty_cache()
        del flush

    if args.cl_steps > 0 and rank == 0 and args.far_field != "direct":
        # CL / CDi history of the benchmarked form against direct all-pairs
        # sweeps (FP32 compensated, within ~1e-7 of FP64 per sweep) from the
        # same seeded initial state, step by step, over one flapping cycle
        # (43 steps) at --cl-particles (the direct sweeps' N^2 cost bounds the
        # size): with the stretching term (the timed step) and without it (the
        # reference's hybrid solver, experiment_hybrid_panel_particle.py:140-143)
        torch.cuda.empty_cache()
        ncl = args.cl_particles
        result["cl_history_vs_direct"] = {}
        for stretch in (True, False):
            hist = {}
            for ff in (args.far_field, "direct"):
                progress(f"CL history, far field {ff}, {ncl} particles, stretching {stretch}")
                st2 = Step(ncl, args.precision, device, far_field=ff, leaf=args.leaf,
                           steps_hint=args.cl_steps, stretch=stretch)
                for _ in range(args.cl_steps):
                    st2.run()
                hist[ff] = (st2.hs.cl.copy(), st2.hs.cdi.copy(), st2.field.np)
                del st2
                torch.cuda.empty_cache()
            ca, da, na = hist[args.far_field]
            cb, db, nb = hist["direct"]
            result["cl_history_vs_direct"]["stretching_on" if stretch else "stretching_off"] = {
                "steps": args.cl_steps, "particles_seeded": ncl, "particles_final": int(nb),
                "cl_err_max_over_max": float(abs(ca - cb).max() / abs(cb).max()),
                "cdi_err_max_over_max": float(abs(da - db).max() / abs(db).max()),
                "cl_abs_err_max": float(abs(ca - cb).max()),
                "cdi_abs_err_max": float(abs(da - db).max()),
                "cl": [float(x) for x in cb], "cdi": [float(x) for x in db]}
        result["cl_history_vs_direct"]["convention"] = (
            "max_k |x_k - ref_k| / max_k |ref_k| over the history (the flapping CL crosses "
            "zero, where a per-step ratio is undefined)")
        result["cl_history_vs_direct"]["reference"] = (
            "direct all-pairs sweeps, FP32 compensated, same seeded state")

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
        if args.sweep_case:
            run_sweep_case(args)
        elif args.impl == "reference":
            run_reference(args, rank, world)
        else:
            run_ours(args, rank, world)
    finally:
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
