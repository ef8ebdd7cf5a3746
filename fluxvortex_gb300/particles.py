"""Device-resident VortexParticleField (mirror of src/fluxvortex/particles.py).

Same public surface as the reference class (particles.py:15-246):
``add_particle``, ``add_particles_batch``, ``positions``/``gammas``/
``sigmas``, ``induce_velocity_at``, ``advect_rk3`` and the Pedrizzetti
relaxation run after every step.  The particle store lives in HBM as
capacity-sized FP64 AoS tensors (pos, gamma, sigma, age, RK3 registers);
every step is a fixed sequence of stream-ordered launches of the C ABI:

  per RK3 stage: velocity sweep -> stage_position -> [stretch sweep ->
  stage_strength];  then finalize (NaN/Inf guard, age) and, if rlxf > 0, a
  vorticity sweep with the Gaussian-erf core (as particles.py:219 always
  uses) -> relax.

``precision="f32c"`` runs the sweeps in FP32 with compensated accumulation;
positions, strengths and the time integration stay FP64.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _capi

RK3_COEFFS = ((0.0, 1.0 / 3.0), (-5.0 / 9.0, 15.0 / 16.0), (-153.0 / 128.0, 8.0 / 15.0))


class VortexParticleField:
    """Structure of FP64 device arrays holding up to ``max_particles`` particles."""

    def __init__(self, max_particles=50000, nu=0.0, rlxf=0.3, kernel="gaussianerf",
                 precision="f64", device="cuda", relax_kernel="gaussianerf", far_field=None,
                 theta=0.5, leaf_target=64):
        self.max_particles = int(max_particles)
        self.nu = float(nu)
        self.rlxf = float(rlxf)
        self.kernel = kernel
        self.relax_kernel = relax_kernel
        self.precision = precision
        self.device = torch.device(device)
        cap = self.max_particles
        z3 = lambda: torch.zeros((cap, 3), dtype=torch.float64, device=self.device)  # noqa: E731
        z1 = lambda: torch.zeros(cap, dtype=torch.float64, device=self.device)  # noqa: E731
        self._pos, self._gamma, self._sigma, self._age = z3(), z3(), z1(), z1()
        self._rk_X, self._rk_G, self._rk_s = z3(), z3(), z1()
        self._u, self._S, self._w = z3(), z3(), z3()
        self._scratch = torch.empty(1, dtype=torch.uint8, device=self.device)
        self.np = 0
        # bumped whenever positions (or the count) change: a tree sweep at
        # the positions of the tree's last build reuses its structure
        self._pos_version = 0
        self._tree_version = -1
        self._lib = _capi.load()
        # Optional profiling hook: when a list, every sweep appends
        # (mode, kernel, n_targets, n_sources, start_event, end_event).
        self.sweep_events = None
        # (mode, kernel, stats, eval_ms, local_ms, validation) when profiling
        self.tree_events = []
        # far_field: the self-sweeps (every particle a target) use the
        # cell-binned treecode with accepted cells evaluated per target particle
        # ("tree" / "m2p"), as analytic local expansions per leaf ("m2l"), or
        # with the learned far-field operator ("learned": analytic translation
        # + the trained network's residual, FP64-validated every sweep); sweeps
        # at other targets stay direct.
        self.tree = None
        self.far_field = far_field or "direct"
        # the per-step FP64 judge of the local-expansion far field: pairs
        # judged on the step's first velocity and stretching sweeps, and the
        # expansion error above which a pair counts as failed (see
        # TreeSweeper.set_validation)
        self.validate_samples = 256
        self.validate_tol = 0.1
        self._validate_next = False
        if far_field in ("tree", "m2p", "m2l", "learned"):
            from .tree import TreeSweeper
            self.tree = TreeSweeper(theta=theta, leaf_target=leaf_target)
            if far_field == "learned":
                from .learned import FarFieldMLP
                self.mlp = FarFieldMLP.load(device=self.device)
                self.tree.set_far_field("learned", mlp=self.mlp)
            elif far_field == "m2l":
                self.tree.set_far_field("m2l")
        elif far_field not in (None, "direct"):
            raise ValueError(f"unknown far_field {far_field!r}")

    # ---- particle management (particles.py:35-66) ----------------------------
    def add_particle(self, X, Gamma, sigma):
        self.add_particles_batch(np.asarray(X, dtype=np.float64).reshape(1, 3),
                                 np.asarray(Gamma, dtype=np.float64).reshape(1, 3),
                                 np.asarray([sigma], dtype=np.float64))

    def add_particles_batch(self, positions, gammas, sigmas):
        n = int(positions.shape[0])
        if self.np + n > self.max_particles:
            raise RuntimeError(
                f"Particle field would overflow ({self.np}+{n} > {self.max_particles})")
        sl = slice(self.np, self.np + n)
        t = lambda a: torch.as_tensor(a, dtype=torch.float64, device=self.device)  # noqa: E731
        self._pos[sl] = t(positions).reshape(n, 3)
        self._gamma[sl] = t(gammas).reshape(n, 3)
        self._sigma[sl] = t(sigmas).reshape(n)
        self._age[sl] = 0.0
        self.np += n
        self._pos_version += 1

    @property
    def positions(self):
        return self._pos[: self.np].cpu().numpy().copy()

    @property
    def gammas(self):
        return self._gamma[: self.np].cpu().numpy().copy()

    @property
    def sigmas(self):
        return self._sigma[: self.np].cpu().numpy().copy()

    @property
    def ages(self):
        return self._age[: self.np].cpu().numpy().copy()

    # ---- snapshot / restore ------------------------------------------------------
    def snapshot(self, host=False):
        """The particle state (positions, strengths, cores, ages of the live
        particles): device copies, or NumPy arrays with ``host``."""
        n = self.np
        st = {k: getattr(self, "_" + k)[:n].clone() for k in ("pos", "gamma", "sigma", "age")}
        if host:
            st = {k: v.cpu().numpy() for k, v in st.items()}
        st["np"] = n
        return st

    def restore(self, st):
        """Puts back a state taken by ``snapshot`` (device or host arrays)."""
        n = int(st["np"])
        if n > self.max_particles:
            raise ValueError(f"snapshot of {n} particles exceeds the capacity {self.max_particles}")
        for k in ("pos", "gamma", "sigma", "age"):
            getattr(self, "_" + k)[:n].copy_(torch.as_tensor(st[k]), non_blocking=False)
        self.np = n
        self._pos_version += 1

    def positions_changed(self):
        """Call after writing the position buffer directly (``_pos``)."""
        self._pos_version += 1

    # ---- population control (newton_pc/adapters/flap.py:466-563) -----------------
    def _pop_scratch_for(self, n):
        nb = self._lib.fvx_vpm_population_scratch_bytes(n)
        if getattr(self, "_pop_scratch", None) is None or self._pop_scratch.numel() < nb:
            self._pop_scratch = torch.empty(int(nb), dtype=torch.uint8, device=self.device)
        return self._pop_scratch

    def drop_oldest(self, keep):
        """Keeps the newest ``keep`` particles; returns how many were dropped."""
        n = self.np
        if n <= keep:
            return 0
        sc = self._pop_scratch_for(n)
        out = ctypes.c_int64(n)
        _capi.check(self._lib.fvx_vpm_drop_oldest(
            n, int(keep), self._pos.data_ptr(), self._gamma.data_ptr(), self._sigma.data_ptr(),
            self._age.data_ptr(), ctypes.byref(out), sc.data_ptr(), sc.numel(), self._stream()))
        self.np = int(out.value)
        self._pos_version += 1
        return n - self.np

    def merge_pass(self, ref_pts, speed, eps=1e-3, protect_newest=64, protect_dist=None):
        """One pass of pairwise moment-conserving merging judged at the wing
        reference points ``ref_pts`` ((R,3), R <= 64) against eps x ``speed``;
        returns the number of merges."""
        ref = np.ascontiguousarray(ref_pts, dtype=np.float64).reshape(-1, 3)
        wing_c = np.ascontiguousarray(ref.mean(axis=0))
        dref = torch.as_tensor(ref, device=self.device)
        n = self.np
        sc = self._pop_scratch_for(max(n, 1))
        out, merged = ctypes.c_int64(n), ctypes.c_int64(0)
        _capi.check(self._lib.fvx_vpm_merge_pass(
            n, self._pos.data_ptr(), self._gamma.data_ptr(), self._sigma.data_ptr(),
            self._age.data_ptr(), dref.data_ptr(), ref.shape[0], wing_c.ctypes.data,
            float(speed), float(eps), int(protect_newest),
            float(protect_dist) if protect_dist else 0.0, ctypes.byref(out),
            ctypes.byref(merged), sc.data_ptr(), sc.numel(), self._stream()))
        if merged.value:
            self.np = int(out.value)
            self._pos_version += 1
        return int(merged.value)

    # ---- sweeps ----------------------------------------------------------------
    def _stream(self):
        return torch.cuda.current_stream(self.device).cuda_stream

    def _ensure_scratch(self, nbytes):
        if self._scratch.numel() < nbytes:
            self._scratch = torch.empty(int(nbytes * 5 // 4) + 256, dtype=torch.uint8,
                                        device=self.device)

    def _sweep(self, mode, tgt, tgt_gamma, n_tgt, out_a, out_b=None, kernel=None):
        lib = self._lib
        pid = _capi.PRECISIONS[self.precision]
        kid = _capi.KERNELS[kernel or self.kernel]
        n = self.np
        nbytes = lib.fvx_particle_pairs_scratch_bytes(mode, pid, n_tgt, n)
        self._ensure_scratch(nbytes)
        ev = None
        if self.sweep_events is not None:
            ev = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
            ev[0].record()
        if (self.tree is not None and tgt is self._pos and n_tgt == n
                and mode in (_capi.PAIR_VELOCITY, _capi.PAIR_STRETCH,
                             _capi.PAIR_VELOCITY_STRETCH, _capi.PAIR_VORTICITY)):
            if self.far_field in ("m2l", "learned"):
                self.tree.set_validation(
                    self.validate_samples if self._validate_next else 0, self.validate_tol)
            stats = self.tree.sweep(mode, kernel or self.kernel, self._pos, self._gamma,
                                    self._sigma, n, out_a, out_b, tgt_gamma=tgt_gamma,
                                    check=ev is not None,
                                    same_positions=self._tree_version == self._pos_version)
            self._tree_version = self._pos_version
            if ev is not None:
                ev[1].record()
                self.sweep_events.append((mode, "tree/" + (kernel or self.kernel), n_tgt, n,
                                          ev[0], ev[1]))
                local = self.far_field in ("m2l", "learned")
                val = self.tree.last_judge() if local and self._validate_next else None
                self.tree_events.append((mode, kernel or self.kernel, stats.copy(),
                                         self.tree.last_eval_ms(),
                                         self.tree.last_local_ms() if local else 0.0,
                                         val if val and val["checked"] else None))
            return
        _capi.check(lib.fvx_particle_pairs(
            mode, kid, pid, tgt.data_ptr(), None if tgt_gamma is None else tgt_gamma.data_ptr(),
            n_tgt, self._pos.data_ptr(), self._gamma.data_ptr(), self._sigma.data_ptr(), n,
            out_a.data_ptr(), None if out_b is None else out_b.data_ptr(),
            self._scratch.data_ptr(), self._scratch.numel(), self._stream()))
        if ev is not None:
            ev[1].record()
            self.sweep_events.append((mode, kernel or self.kernel, n_tgt, n, ev[0], ev[1]))

    def induce_velocity_at(self, target_points):
        """Velocity induced by all particles at target points (particles.py:72)."""
        is_t = isinstance(target_points, torch.Tensor)
        if self.np == 0:
            return torch.zeros_like(target_points) if is_t else np.zeros_like(target_points)
        t = torch.as_tensor(target_points, dtype=torch.float64, device=self.device).contiguous()
        M = t.shape[0]
        u = torch.empty((M, 3), dtype=torch.float64, device=self.device)
        self._sweep(_capi.PAIR_VELOCITY, t, None, M, u)
        return u if is_t else u.cpu().numpy()

    # ---- RK3 + rVPM (particles.py:85-199) --------------------------------------
    def _extra_velocity(self, fn, n):
        if fn is None:
            return None
        v = fn(self._pos[:n])
        return torch.as_tensor(v, dtype=torch.float64, device=self.device).reshape(n, 3).contiguous()

    def advect_rk3(self, dt, U_inf_func, bound_velocity_func=None, stretch=True, free_wake=True):
        """Advance one time step.  ``U_inf_func`` is either a constant freestream
        3-vector (kept on the device path) or a callable X -> (N,3) as in the
        reference; ``bound_velocity_func`` likewise (callable or None)."""
        n = self.np
        if n == 0:
            return
        lib, st = self._lib, self._stream()
        dt = float(dt)
        if callable(U_inf_func):
            u_inf_host = np.zeros(3)
            inf_fn = U_inf_func
        else:
            u_inf_host = np.ascontiguousarray(U_inf_func, dtype=np.float64).reshape(3)
            inf_fn = None
        for stage, (a, b) in enumerate(RK3_COEFFS):
            if free_wake:
                # the FP64 judge of the local-expansion far field runs on the
                # step's first velocity and first stretching sweeps; the sweeps
                # in between keep its per-class decisions
                self._validate_next = stage == 0
                self._sweep(_capi.PAIR_VELOCITY, self._pos, None, n, self._u)
                self._validate_next = False
            extra = None
            if inf_fn is not None or bound_velocity_func is not None:
                eb = self._extra_velocity(bound_velocity_func, n)
                ei = self._extra_velocity(inf_fn, n)
                extra = eb if ei is None else (ei if eb is None else eb + ei)
            _capi.check(lib.fvx_vpm_stage_position(
                n, a, b, dt, u_inf_host.ctypes.data, self._u.data_ptr() if free_wake else None,
                None if extra is None else extra.data_ptr(), self._pos.data_ptr(),
                self._rk_X.data_ptr(), st))
            self._pos_version += 1
            if stretch:
                self._validate_next = stage == 0
                self._sweep(_capi.PAIR_STRETCH, self._pos, self._gamma, n, self._S)
                self._validate_next = False
                _capi.check(lib.fvx_vpm_stage_strength(
                    n, a, b, dt, self.nu, self._S.data_ptr(), self._gamma.data_ptr(),
                    self._sigma.data_ptr(), self._rk_G.data_ptr(), self._rk_s.data_ptr(), st))
        _capi.check(lib.fvx_vpm_finalize(n, dt, self._pos.data_ptr(), self._gamma.data_ptr(),
                                         self._age.data_ptr(), st))
        self._relax_pedrizzetti()

    def _relax_pedrizzetti(self):
        """particles.py:202-246; the vorticity uses ``relax_kernel``
        (Gaussian-erf, as the reference always does)."""
        n = self.np
        if self.rlxf <= 0 or n == 0:
            return
        self._sweep(_capi.PAIR_VORTICITY, self._pos, None, n, self._w, kernel=self.relax_kernel)
        _capi.check(self._lib.fvx_vpm_relax(n, self.rlxf, self._w.data_ptr(),
                                            self._gamma.data_ptr(), self._stream()))

