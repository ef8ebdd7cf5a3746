"""Batched aeroelastic flutter sweep (Goland wing) on one GPU.

The reference couples PteraSoftware's UVLM with its beam FE per airspeed,
one airspeed at a time (src/fluxvortex/aeroelastic_solver.py:68-221,
tests/benchmark_goland.py:100-248).  Here every airspeed of the sweep is an
independent environment of one persistent kernel (fvx_flutter_sweep): one
CTA per environment runs that environment's whole time history -- beam
deformation of the lattice, AIC, wake and particle induction, the FP64 LU
solve, Kutta-Joukowski loads, station lift and torque, the Newmark beam
step, ring shedding and particle conversion -- with its state in shared and
global memory, so environments with different step counts (uneven wake
lengths) finish independently.

Model (PteraSoftware-free; the same in the CPU oracle):
  * flat rectangular wing (NACA 0012 mean line), chord c, semi-span b, nc x ns
    uniform panels, clamped root at y = 0; freestream V (cos a, 0, sin a);
  * beam node displacements w and twist theta (nose up) interpolated
    linearly at each vertex's span station; a vertex at chordwise x moves to
    (x_ea + (x - x_ea) cos theta, y, w - (x - x_ea) sin theta), x_ea at
    33 % chord; the motion's velocity enters the boundary condition and the
    loads (the reference mutates vertices only, aeroelastic_solver.py:150-221);
  * station lift = sum of the panel forces' z components per spanwise
    column, station torque = sum of F_z (x_ea - x) about the elastic axis
    (the reference takes the arm from x = 0, :131-134), both distributed
    linearly to the beam nodes (beam_fe.py:316-351);
  * the last n_keep ring rows stay rings; older rows become 4 particles per
    ring (Winckelmans core, sigma = 1.3 x mean edge) convected with the
    freestream; each environment keeps its newest max_particles particles;
  * tip perturbation w = 0.05 m, theta = 2 deg, a0 = M^-1 (-K d0)
    (benchmark_goland.py:111-121).
Flutter: envelope growth rate of the tip heave history
(benchmark_goland.py:66-97) per airspeed; the flutter speed is the first
sign change from decay to growth, linearly interpolated (:221-229).
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass, field

import numpy as np

from .beam import NEWMARK_BETA, NEWMARK_GAMMA, BeamModel
from .geometry import rectangular_wing


@dataclass
class FlutterConfig:
    chord: float = 1.8288
    semi_span: float = 6.096
    nc: int = 4
    ns: int = 8
    alpha_deg: float = 2.0
    rho: float = 1.225
    nu: float = 15.06e-6
    dt: float = 0.003
    num_chords: float = 100.0
    x_ea: float = 0.33               # elastic axis, fraction of chord from the LE
    rc0: float = 0.03 * 1.8288       # ring core radius
    n_keep: int = 10
    max_particles: int = 2048
    tip_w: float = 0.05
    tip_theta_deg: float = 2.0
    # "physical": the model above (motion velocity in the boundary condition,
    # torque about the elastic axis, deformation at every vertex); "reference":
    # the reference's own coupling (aeroelastic_solver.py:68-221): the station
    # lift's moment about x = 0 with the collocation point's arm, vertices
    # mutated per panel at its collocation span station, no motion velocity,
    # coupling from step 1 on
    coupling: str = "physical"
    beam: dict = field(default_factory=lambda: dict(
        length=6.096, n_elements=8, EI=9.773e6, GJ=0.988e6, m_per_length=35.72,
        Ip=35.72 * 1.8288 ** 2 / 24.0, x_ea_cg=0.10 * 1.8288, structural_damping=0.005))

    def velocities(self, n=64, lo=80.0, hi=180.0):
        return np.linspace(lo, hi, n)

    def n_steps(self, V):
        return int(math.ceil(self.num_chords * self.chord / (V * self.dt)))

    def u_inf(self, V):
        a = math.radians(self.alpha_deg)
        return np.array([V * math.cos(a), 0.0, V * math.sin(a)])

    def base_vertices(self):
        return rectangular_wing(self.chord, self.semi_span, self.nc, self.ns, symmetric=False)

    def beam_model(self):
        return BeamModel(**self.beam)


def goland(**kw):
    return FlutterConfig(**kw)


def envelope_growth(signal, dt):
    """Exponential growth rate (1/s) of |signal|'s peaks: a least-squares line
    through log(peak) against time, skipping the first peak when there are
    more than four (benchmark_goland.py:66-97)."""
    s = np.abs(np.asarray(signal, dtype=np.float64))
    if s.size < 10:
        return 0.0
    i = np.flatnonzero((s[1:-1] > s[:-2]) & (s[1:-1] > s[2:])) + 1
    if i.size < 3:
        return 0.0
    t = i * dt
    a = np.maximum(s[i], 1e-15)
    if i.size > 4:
        t, a = t[1:], a[1:]
    return float(np.polyfit(t, np.log(a), 1)[0])


def flutter_speed(velocities, sigma):
    """First decay -> growth crossing of sigma(V), linearly interpolated."""
    order = np.argsort(velocities)
    V = np.asarray(velocities, dtype=np.float64)[order]
    s = np.asarray(sigma, dtype=np.float64)[order]
    for k in range(len(V) - 1):
        if s[k] < 0 < s[k + 1]:
            return float(V[k] - s[k] * (V[k + 1] - V[k]) / (s[k + 1] - s[k]))
    return None


def interp_weights(y_query, y_nodes):
    """(index, fraction) of linear interpolation at y_query (clamped)."""
    k = np.clip(np.searchsorted(y_nodes, y_query, side="right") - 1, 0, len(y_nodes) - 2)
    xi = np.clip((y_query - y_nodes[k]) / (y_nodes[k + 1] - y_nodes[k]), 0.0, 1.0)
    return k.astype(np.int64), xi


__all__ = ["FlutterConfig", "goland", "envelope_growth", "flutter_speed", "NEWMARK_BETA",
           "NEWMARK_GAMMA"]


# ---- device sweep ----------------------------------------------------------------


class _Params(ctypes.Structure):
    _fields_ = [("n_env", ctypes.c_int), ("nc", ctypes.c_int), ("ns", ctypes.c_int),
                ("nnodes", ctypes.c_int), ("n_keep", ctypes.c_int),
                ("max_particles", ctypes.c_int), ("max_steps", ctypes.c_int),
                ("coupling", ctypes.c_int),
                ("x_ea", ctypes.c_double), ("rc0", ctypes.c_double), ("nu", ctypes.c_double),
                ("rho", ctypes.c_double), ("dt", ctypes.c_double), ("beta", ctypes.c_double),
                ("gamma", ctypes.c_double), ("pad1", ctypes.c_double)] + [
        (n, ctypes.c_void_p) for n in ("base_verts", "vert_node", "vert_xi", "station_node",
                                       "station_xi", "kinv", "mr", "cr", "u_inf", "n_steps")]


class _State(ctypes.Structure):
    _fields_ = [(n, ctypes.c_void_p) for n in (
        "d", "v", "a", "W", "wgam", "wage", "nrows", "ppos", "palp", "psig", "phead", "pcount",
        "gprev", "has_prev", "hist_w", "hist_th", "step", "gd", "hist_nodes")]


COUPLINGS = {"physical": 0, "reference": 1}


def deform_vertices(cfg, beam, d, base=None):
    """Host copy of the kernel's deformation (initial wake row only)."""
    base = cfg.base_vertices() if base is None else base
    y = base[..., 1]
    w = np.interp(y, beam.y_nodes, d[0::3])
    th = np.interp(y, beam.y_nodes, d[2::3])
    x_ea = cfg.x_ea * cfg.chord
    xr = base[..., 0] - x_ea
    out = base.copy()
    out[..., 0] = x_ea + xr * np.cos(th)
    out[..., 2] = base[..., 2] + w - xr * np.sin(th)
    return out


class FlutterSweep:
    """All airspeeds of a sweep as environments of the persistent kernel.

    ``run()`` advances every environment to its own step count (one launch,
    or ``chunk`` steps per launch, optionally captured once in a CUDA graph
    and replayed); ``sigma()`` and ``flutter_speed()`` post-process the tip
    histories on the host."""

    def __init__(self, cfg: FlutterConfig, velocities, precision="f64", threads=None,
                 device="cuda", node_histories=False):
        import torch
        from . import _capi
        from .geometry import lattice
        self.torch = torch
        self.capi = _capi
        self.lib = _capi.load()
        self.cfg = cfg
        self.V = np.asarray(velocities, dtype=np.float64)
        self.precision = _capi.PRECISIONS[precision]
        self.device = torch.device(device)
        E = len(self.V)
        nc, ns = cfg.nc, cfg.ns
        P = nc * ns
        self.threads = None if threads in (None, "auto") else int(threads)
        beam = cfg.beam_model()
        self.beam = beam
        self.steps = np.array([cfg.n_steps(v) for v in self.V], dtype=np.int32)
        self.max_steps = int(self.steps.max())
        base = cfg.base_vertices()
        vn, vx = interp_weights(base[..., 1].reshape(-1), beam.y_nodes)
        y_st = (np.arange(ns) + 0.5) * cfg.semi_span / ns
        sn, sx = interp_weights(y_st, beam.y_nodes)
        kinv = beam.newmark_inverse(cfg.dt)
        f64 = lambda a: torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64),  # noqa: E731
                                        device=self.device)
        i32 = lambda a: torch.as_tensor(np.ascontiguousarray(a, dtype=np.int32),  # noqa: E731
                                        device=self.device)
        self._keep = dict(
            base=f64(base.reshape(-1, 3)), vn=i32(vn), vx=f64(vx), sn=i32(sn), sx=f64(sx),
            kinv=f64(kinv), mr=f64(beam.Mr), cr=f64(beam.Cr),
            u=f64(np.stack([cfg.u_inf(v) for v in self.V])), ns=i32(self.steps))
        k = self._keep
        self.params = _Params(
            n_env=E, nc=nc, ns=ns, nnodes=beam.nnodes, n_keep=cfg.n_keep,
            max_particles=cfg.max_particles, max_steps=self.max_steps,
            coupling=COUPLINGS[cfg.coupling],
            x_ea=cfg.x_ea * cfg.chord, rc0=cfg.rc0, nu=cfg.nu, rho=cfg.rho, dt=cfg.dt,
            beta=NEWMARK_BETA, gamma=NEWMARK_GAMMA, pad1=0.0,
            base_verts=k["base"].data_ptr(), vert_node=k["vn"].data_ptr(),
            vert_xi=k["vx"].data_ptr(), station_node=k["sn"].data_ptr(),
            station_xi=k["sx"].data_ptr(), kinv=k["kinv"].data_ptr(), mr=k["mr"].data_ptr(),
            cr=k["cr"].data_ptr(), u_inf=k["u"].data_ptr(), n_steps=k["ns"].data_ptr())
        if cfg.coupling not in COUPLINGS:
            raise ValueError(f"coupling must be one of {sorted(COUPLINGS)}, not {cfg.coupling!r}")
        # initial state: tip perturbation, a0 = M^-1 (-K d0), first wake row at
        # the TE (of the undeformed wing with the reference's coupling, which
        # shapes the wing from the first coupling on)
        d0, v0, a0 = beam.initial_state(cfg.tip_w, np.radians(cfg.tip_theta_deg))
        te = lattice(base if cfg.coupling == "reference"
                     else deform_vertices(cfg, beam, d0, base)).te_back
        ndof = beam.ndof
        Pm = cfg.max_particles
        self._init = dict(d=np.tile(d0, (E, 1)), v=np.tile(v0, (E, 1)), a=np.tile(a0, (E, 1)),
                          te=te)
        z = lambda *s: torch.zeros(s, dtype=torch.float64, device=self.device)  # noqa: E731
        zi = lambda *s: torch.zeros(s, dtype=torch.int32, device=self.device)  # noqa: E731
        self.st = dict(d=z(E, ndof), v=z(E, ndof), a=z(E, ndof),
                       W=z(E, cfg.n_keep + 2, ns + 1, 3), wgam=z(E, cfg.n_keep + 1, ns),
                       wage=z(E, cfg.n_keep + 1), nrows=zi(E), ppos=z(E, Pm, 3),
                       palp=z(E, Pm, 3), psig=z(E, Pm), phead=zi(E), pcount=zi(E),
                       gprev=z(E, P), has_prev=zi(E), hist_w=z(E, self.max_steps),
                       hist_th=z(E, self.max_steps), step=zi(E), gd=z(E, ndof))
        if node_histories:
            # every beam node's heave and twist per recorded step
            self.st["hist_nodes"] = z(E, self.max_steps, beam.nnodes, 2)
        self.state = _State(**{n: t.data_ptr() for n, t in self.st.items()})
        self._graph = None
        self.reset()
        if self.threads is None:
            self.threads = self.autotune()

    def autotune(self, steps=40):
        """Threads per environment CTA (the number of slices the wake sums are
        split into) from timing the first ``steps`` steps of this sweep with
        each candidate; cached per device and problem."""
        from . import autotune
        P = self.cfg.nc * self.cfg.ns
        cands = [t for t in (64, 128, 256, 512) if t >= 2 * P and t % (2 * P) == 0]
        st = self.torch.cuda.current_stream(self.device).cuda_stream

        def run(t):
            self.reset()
            self.threads = t
            self._launch(min(steps, self.max_steps), st)

        key = (f"flutter_sweep/nc{self.cfg.nc}ns{self.cfg.ns}/E{len(self.V)}"
               f"/particles{self.cfg.max_particles}/prec{self.precision}/steps{steps}")
        best = autotune.best(key, cands, run)
        self.reset()
        return best

    def reset(self):
        torch = self.torch
        for t in self.st.values():
            t.zero_()
        self.st["d"].copy_(torch.as_tensor(self._init["d"]))
        self.st["v"].copy_(torch.as_tensor(self._init["v"]))
        self.st["a"].copy_(torch.as_tensor(self._init["a"]))
        self.st["W"][:, 0] = torch.as_tensor(self._init["te"], device=self.device)

    def _launch(self, step_end, stream):
        self.capi.check(self.lib.fvx_flutter_sweep(ctypes.addressof(self.params),
                                                   ctypes.addressof(self.state), int(step_end),
                                                   self.precision, self.threads, stream))

    def run(self, chunk=None, graph=False):
        """Advances every environment to its last step.  chunk: steps per launch
        (default: all in one launch).  graph: capture the launches once in a
        CUDA graph and replay it (the state must be reset before a replay)."""
        torch = self.torch
        chunk = chunk or self.max_steps
        ends = list(range(chunk, self.max_steps, chunk)) + [self.max_steps]
        if not graph:
            st = torch.cuda.current_stream(self.device).cuda_stream
            for e in ends:
                self._launch(e, st)
            return
        if self._graph is None:
            s = torch.cuda.Stream(device=self.device)
            s.wait_stream(torch.cuda.current_stream(self.device))
            g = torch.cuda.CUDAGraph()
            with torch.cuda.stream(s):
                # the kernel's one-time attribute setup happens outside capture
                self._launch(0, s.cuda_stream)
                g.capture_begin()
                for e in ends:
                    self._launch(e, s.cuda_stream)
                g.capture_end()
            torch.cuda.current_stream(self.device).wait_stream(s)
            self._graph = g
        self._graph.replay()

    def histories(self):
        """Tip heave and twist per environment: one sample per step, or with
        the reference's coupling one per coupled step (n_steps - 2)."""
        w = self.st["hist_w"].cpu().numpy()
        th = self.st["hist_th"].cpu().numpy()
        n = self.steps - (2 if self.cfg.coupling == "reference" else 0)
        return ([w[e, :n[e]] for e in range(len(self.V))],
                [th[e, :n[e]] for e in range(len(self.V))])

    def node_histories(self, env):
        """(w, theta) of every beam node per recorded step of environment
        ``env``: two (steps, nnodes) arrays (needs node_histories=True)."""
        if "hist_nodes" not in self.st:
            raise ValueError("the sweep was made without node_histories=True")
        n = int(self.steps[env]) - (2 if self.cfg.coupling == "reference" else 0)
        h = self.st["hist_nodes"][env, :n].cpu().numpy()
        return h[..., 0].copy(), h[..., 1].copy()

    def sigma(self):
        w, _ = self.histories()
        return np.array([envelope_growth(x, self.cfg.dt) for x in w])

    def flutter_speed(self):
        return flutter_speed(self.V, self.sigma())
