"""Device-resident hybrid panel-particle step (mirror of the reference's HybridSolver).

One ``HybridStep.step()`` runs, on the GPU and in the order of the
reference's solver (tests/experiment_hybrid_panel_particle.py:87-204 on top
of PteraSoftware's step):

  kinematics -> lattice -> AIC (expanded ring Biot-Savart . n) ->
  wake on collocation (ring rows + particles) -> rhs -> FP64 LU solve ->
  loads (bound legs, CL / CDi) -> shed + convect the ring wake ->
  rows >= N_keep to particles -> particle RK3 (VortexParticleField)

Every stage is a C-ABI kernel over device arrays; the host keeps only the
wake row count and reads the particle count once per step.  Particle sweeps
run in FP64 or FP32-compensated (``precision``); the panel side, the AIC
solve and the time integration stay FP64.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _capi
from .geometry import HybridConfig
from .particles import VortexParticleField


class HybridStep:
    def __init__(self, cfg: HybridConfig, precision: str = "f64", device="cuda"):
        self.cfg = cfg
        self.precision = precision
        self.device = torch.device(device)
        self.lib = _capi.load()
        col, surf, kins = cfg.layout()
        nc, ns, w = cfg.verts.shape[0] - 1, int(col.size), cfg.verts.shape[1]
        self.nc, self.ns, self.w, self.P = nc, ns, w, nc * ns
        d = dict(dtype=torch.float64, device=self.device)
        P = self.P
        # surface layout: strip -> vertex column, column -> surface, motions
        i32 = dict(dtype=torch.int32, device=self.device)
        self._col = torch.as_tensor(np.asarray(col, dtype=np.int32), **i32)
        self._surf = torch.as_tensor(np.asarray(surf, dtype=np.int32), **i32)
        self._motion = torch.tensor([[k.heave_amp, k.flap_amp, 2.0 * np.pi / k.period, k.y0]
                                     for k in kins], **d).reshape(-1).contiguous()
        self._sf = _capi.Surfaces(ns, w, self._col.data_ptr(), self._surf.data_ptr(),
                                  self._motion.data_ptr())
        self.sf = ctypes.addressof(self._sf)
        self.base = torch.as_tensor(cfg.verts.reshape(-1, 3), **d).contiguous()
        self.verts = torch.empty_like(self.base)
        self.verts_next = torch.empty_like(self.base)
        z3 = lambda n: torch.zeros((n, 3), **d)  # noqa: E731
        self.L = {k: z3(P) for k in ("br", "fr", "fl", "bl", "normal", "leg_vec")}
        # collocation points and bound-leg centres side by side, so that the
        # wake rings and the particles are swept at both in one call
        self._pts = z3(2 * P)
        self.L["colloc"], self.L["leg_center"] = self._pts[:P], self._pts[P:]
        self.L["area"] = torch.zeros(P, **d)
        self.te = z3(w)
        self.te_next = z3(w)
        self.Ln = {k: z3(P) for k in self.L if k != "area"}
        self.Ln["area"] = torch.zeros(P, **d)
        self.aic = torch.zeros((P, P), **d)
        # P <= 192: the AIC is factorised on a side stream while the wake and
        # the particles are swept at the collocation points, and the solve
        # waits for it (the same strengths bit for bit as the fused solve)
        wb = int(self.lib.fvx_lu_workspace_bytes(P))
        self._lu_work = torch.empty(wb // 8, **d) if wb > 0 else None
        self._lu_side = torch.cuda.Stream(self.device) if wb > 0 else None
        self.rhs = torch.zeros(P, **d)
        self.gamma = torch.zeros(P, **d)
        self.gamma_prev = torch.zeros(P, **d)
        self.force = z3(P)
        # ring wake: vertex lattice (R+1 rows) ping-pong, row strengths, ages
        rows = cfg.n_keep + 2
        self.W = [z3(rows * w), z3(rows * w)]
        self.wg = [torch.zeros(rows * ns, **d), torch.zeros(rows * ns, **d)]
        self.wa = [torch.zeros(rows, **d), torch.zeros(rows, **d)]
        # velocities induced at the wake vertices (free ring wake)
        self._wv = [z3(rows * w) for _ in range(3)] if cfg.free_ring_wake else None
        self.cur = 0
        self.R = 0
        nr = (cfg.n_keep + 1) * ns
        self.wr = {k: z3(nr) for k in ("br", "fr", "fl", "bl")}
        self.wr_s = torch.zeros(nr, **d)
        self.wr_rc = torch.zeros(nr, **d)
        self.wr_age = torch.zeros(nr, **d)
        self._v_ring, self._v_part = z3(2 * P), z3(2 * P)
        self.v_ring_c, self.v_ring_l = self._v_ring[:P], self._v_ring[P:]
        self.v_part_c, self.v_part_l = self._v_part[:P], self._v_part[P:]
        self.v_bound_l = z3(P)
        self.seg_scratch = torch.empty(1, dtype=torch.uint8, device=self.device)
        self.field = VortexParticleField(cfg.max_particles, nu=cfg.nu, rlxf=cfg.rlxf,
                                         kernel=cfg.kernel, precision=precision, device=device,
                                         far_field=cfg.far_field)
        self.count = torch.zeros(1, dtype=torch.int64, device=self.device)
        self.u_inf = np.ascontiguousarray(cfg.u_inf, dtype=np.float64)
        self.s_ref = -1.0 if cfg.s_ref is None else float(cfg.s_ref)
        self.cl_hist = torch.zeros(0, **d)
        self._cl = torch.zeros(4096, **d)
        self._cdi = torch.zeros(4096, **d)
        self.k = 0
        self.n_merged = 0
        self.n_dropped = 0
        if cfg.loads not in ("kj", "bernoulli"):
            raise ValueError(f"loads must be kj or bernoulli, not {cfg.loads!r}")
        if cfg.population not in ("none", "drop", "merge"):
            raise ValueError(f"population must be none, drop or merge, not {cfg.population!r}")
        # initial wake lattice: the trailing edge at t = 0
        self._kin(0.0, self.verts)
        self._lattice(self.verts, self.L, self.te)
        self.W[0][:w].copy_(self.te)

    # ---- helpers ------------------------------------------------------------
    def _st(self):
        return torch.cuda.current_stream(self.device).cuda_stream

    def _kin(self, t, out):
        _capi.check(self.lib.fvx_uvlm_kinematics(self.nc, self.sf, self.base.data_ptr(), t,
                                                 out.data_ptr(), self._st()))

    def _lattice(self, verts, L, te):
        _capi.check(self.lib.fvx_uvlm_lattice(
            verts.data_ptr(), self.nc, self.sf, L["br"].data_ptr(), L["fr"].data_ptr(),
            L["fl"].data_ptr(), L["bl"].data_ptr(),
            L["colloc"].data_ptr() if "colloc" in L else None,
            L["normal"].data_ptr(), L["area"].data_ptr(), L["leg_center"].data_ptr(),
            L["leg_vec"].data_ptr(), te.data_ptr(), self._st()))

    def _rings_at(self, pts, n_pts, out, strengths, n_rings, corners, rc0s, ages):
        """Collapsed ring Biot-Savart of n_rings rings at n_pts points -> out."""
        lib = self.lib
        nb = lib.fvx_segments_collapsed_scratch_bytes(n_pts, n_rings, _capi.LEGS_RING)
        if self.seg_scratch.numel() < nb:
            self.seg_scratch = torch.empty(nb + 256, dtype=torch.uint8, device=self.device)
        _capi.check(lib.fvx_segments_collapsed(
            pts.data_ptr(), n_pts, corners["br"].data_ptr(), corners["fr"].data_ptr(),
            corners["fl"].data_ptr(), corners["bl"].data_ptr(), strengths.data_ptr(),
            rc0s.data_ptr(), None if ages is None else ages.data_ptr(), self.cfg.nu, n_rings,
            _capi.LEGS_RING, out.data_ptr(), None, self.seg_scratch.data_ptr(),
            self.seg_scratch.numel(), self._st()))

    # ---- one step -----------------------------------------------------------
    def panel_loads(self, precision=None):
        """Stages 1-5 (AIC, wake on collocation, solve, loads) at the current
        state without advancing it; returns (CL, CDi).  ``precision``
        overrides the particle sweeps' precision for this evaluation."""
        old = self.field.precision
        if precision is not None:
            self.field.precision = precision
        try:
            self._panel(self._tmp_cl())
        finally:
            self.field.precision = old
        v = self._tmp.cpu().numpy()
        return float(v[0]), float(v[1])

    def _tmp_cl(self):
        if not hasattr(self, "_tmp"):
            self._tmp = torch.zeros(2, dtype=torch.float64, device=self.device)
        return self._tmp

    def step(self):
        k = self.k
        if k >= self._cl.numel():
            self._cl = torch.cat([self._cl, torch.zeros_like(self._cl)])
            self._cdi = torch.cat([self._cdi, torch.zeros_like(self._cdi)])
        self._panel(None)
        self._advance()

    def _panel(self, out2):
        cfg, lib, st = self.cfg, self.lib, self._st()
        P, ns = self.P, self.ns
        t = self.k * cfg.dt
        self._kin(t, self.verts)
        self._lattice(self.verts, self.L, self.te)
        L = self.L
        # 1. AIC
        _capi.check(lib.fvx_uvlm_aic(1, P, L["colloc"].data_ptr(), L["normal"].data_ptr(),
                                     L["br"].data_ptr(), L["fr"].data_ptr(), L["fl"].data_ptr(),
                                     L["bl"].data_ptr(), cfg.rc0, cfg.nu, self.aic.data_ptr(), st))
        fac_done = None
        if self._lu_work is not None:
            aic_ready = torch.cuda.Event()
            aic_ready.record(torch.cuda.current_stream(self.device))
            self._lu_side.wait_event(aic_ready)
            _capi.check(lib.fvx_lu_factor_batched(1, P, self.aic.data_ptr(),
                                                  self._lu_work.data_ptr(),
                                                  self._lu_side.cuda_stream))
            fac_done = torch.cuda.Event()
            fac_done.record(self._lu_side)
        # 2-3. wake on collocation: ring rows + particles
        R = self.R
        Wc, gc, ac = self.W[self.cur], self.wg[self.cur], self.wa[self.cur]
        nr = R * ns
        if R:
            _capi.check(lib.fvx_uvlm_wake_rings(R, self.sf, Wc.data_ptr(), gc.data_ptr(),
                                                ac.data_ptr(),
                                                cfg.rc0, self.wr["br"].data_ptr(),
                                                self.wr["fr"].data_ptr(), self.wr["fl"].data_ptr(),
                                                self.wr["bl"].data_ptr(), self.wr_s.data_ptr(),
                                                self.wr_rc.data_ptr(), self.wr_age.data_ptr(), st))
            # wake rings at the collocation points and the bound-leg centres
            self._rings_at(self._pts, 2 * P, self._v_ring, self.wr_s, nr, self.wr, self.wr_rc,
                           self.wr_age)
        npart = self.field.np
        if npart:
            # the particles at both point sets (the state does not change
            # until the step's convection)
            self.field._sweep(_capi.PAIR_VELOCITY, self._pts, None, 2 * P, self._v_part)
        _capi.check(lib.fvx_uvlm_rhs(self.nc, self.sf, L["colloc"].data_ptr(),
                                     L["normal"].data_ptr(),
                                     self.v_ring_c.data_ptr() if R else None,
                                     self.v_part_c.data_ptr() if npart else None,
                                     self.u_inf.ctypes.data, t, self.rhs.data_ptr(), st))
        # 4. strengths (in place: rhs -> Gamma)
        self.gamma.copy_(self.rhs)
        if fac_done is not None:
            torch.cuda.current_stream(self.device).wait_event(fac_done)
            _capi.check(lib.fvx_lu_solve_factored_batched(1, P, self._lu_work.data_ptr(),
                                                          self.gamma.data_ptr(), st))
        else:
            _capi.check(lib.fvx_lu_solve_batched(1, P, self.aic.data_ptr(),
                                                 self.gamma.data_ptr(), st))
        # 5. loads at the bound-leg centres (wake and particles swept above)
        k = self.k
        cl_p = self._cl[k:].data_ptr() if out2 is None else out2[0:].data_ptr()
        cdi_p = self._cdi[k:].data_ptr() if out2 is None else out2[1:].data_ptr()
        if cfg.loads == "bernoulli":
            # unsteady Bernoulli pressure (flap.py:357-377) from the collocation
            # velocities already swept for the right-hand side
            _capi.check(lib.fvx_uvlm_loads_bernoulli(
                self.nc, self.sf, self.verts.data_ptr(), self.gamma.data_ptr(),
                self.gamma_prev.data_ptr() if k else None, L["colloc"].data_ptr(),
                L["area"].data_ptr(), L["normal"].data_ptr(),
                self.v_ring_c.data_ptr() if R else None,
                self.v_part_c.data_ptr() if npart else None, self.u_inf.ctypes.data, cfg.rho,
                cfg.dt, t, self.s_ref, cl_p, cdi_p, self.force.data_ptr(), st))
            return
        self._rings_at(L["leg_center"], P, self.v_bound_l, self.gamma, P, L,
                       self._rc0_bound(), None)
        _capi.check(lib.fvx_uvlm_loads(
            self.nc, self.sf, self.gamma.data_ptr(), self.gamma_prev.data_ptr() if k else None,
            L["leg_center"].data_ptr(), L["leg_vec"].data_ptr(), L["area"].data_ptr(),
            L["normal"].data_ptr(), self.v_ring_l.data_ptr() if R else None,
            self.v_part_l.data_ptr() if npart else None, self.v_bound_l.data_ptr(),
            self.u_inf.ctypes.data, cfg.rho, cfg.dt, t, self.s_ref, cl_p, cdi_p,
            self.force.data_ptr(), st))

    def _advance(self):
        cfg, lib, st = self.cfg, self.lib, self._st()
        t = self.k * cfg.dt
        R = self.R
        Wc, gc, ac = self.W[self.cur], self.wg[self.cur], self.wa[self.cur]
        # 6. next wake: trailing edge at t + dt, convected rows
        self._kin(t + cfg.dt, self.verts_next)
        self._lattice(self.verts_next, self.Ln, self.te_next)
        nxt = 1 - self.cur
        vel = (None, None, None)
        if cfg.free_ring_wake:
            # free ring wake: every old vertex moves with the velocity the bound
            # rings, the wake rings and the particles induce there (PS core law)
            nv = (R + 1) * self.w
            vb, vw, vp = (t_[:nv] for t_ in self._wv)
            self._rings_at(Wc, nv, vb, self.gamma, self.P, self.L, self._rc0_bound(), None)
            if R:
                self._rings_at(Wc, nv, vw, self.wr_s, R * self.ns, self.wr, self.wr_rc,
                               self.wr_age)
            if self.field.np:
                self.field._sweep(_capi.PAIR_VELOCITY, Wc, None, nv, vp)
            vel = (vb.data_ptr(), vw.data_ptr() if R else None,
                   vp.data_ptr() if self.field.np else None)
        _capi.check(lib.fvx_uvlm_shed(R, self.nc, self.sf, Wc.data_ptr(), gc.data_ptr(),
                                      ac.data_ptr(),
                                      self.te_next.data_ptr(), self.gamma.data_ptr(),
                                      self.u_inf.ctypes.data, cfg.dt, *vel,
                                      self.W[nxt].data_ptr(),
                                      self.wg[nxt].data_ptr(), self.wa[nxt].data_ptr(), st))
        self.cur = nxt
        R += 1
        # 7. rows >= N_keep -> particles
        if R > cfg.n_keep:
            f = self.field
            self.count.fill_(f.np)
            _capi.check(lib.fvx_uvlm_convert(
                R, cfg.n_keep, self.sf, self.W[nxt].data_ptr(), self.wg[nxt].data_ptr(),
                1 if cfg.sigma_rule == "edge" else 0, cfg.speed * cfg.dt, f.max_particles,
                self.count.data_ptr(), f._pos.data_ptr(), f._gamma.data_ptr(),
                f._sigma.data_ptr(), f._age.data_ptr(), st))
            f.np = int(self.count.item())
            f.positions_changed()
            R = cfg.n_keep
        self.R = R
        # 8. particles
        if self.field.np:
            self.field.advect_rk3(cfg.dt, self.u_inf, stretch=cfg.stretch,
                                  free_wake=cfg.free_vpm)
        # 9. population control (flap.py:469-475)
        if cfg.population == "drop" and self.field.np > cfg.pop_max:
            self.n_dropped += self.field.drop_oldest(cfg.pop_max)
        elif cfg.population == "merge" and self.field.np:
            ref = cfg.ref_points(self.L["colloc"]).cpu().numpy()
            self.n_merged += self.field.merge_pass(ref, cfg.speed, cfg.merge_eps,
                                                   cfg.merge_protect, cfg.merge_protect_dist)
        self.gamma_prev.copy_(self.gamma)
        self.k += 1

    # ---- snapshot / restore ------------------------------------------------------
    def snapshot(self, host=False):
        """Everything a later step reads: the ring wake (vertex rows, strengths,
        ages), the last strengths, the step count and CL / CDi history, and the
        particle field.  Device copies, or NumPy arrays with ``host`` (e.g. for
        ``numpy.savez``); ``restore`` resumes bitwise."""
        cur = self.cur
        st = {"W": self.W[cur].clone(), "wg": self.wg[cur].clone(), "wa": self.wa[cur].clone(),
              "gamma": self.gamma.clone(), "gamma_prev": self.gamma_prev.clone(),
              "cl": self._cl[: self.k].clone(), "cdi": self._cdi[: self.k].clone()}
        if host:
            st = {k: v.cpu().numpy() for k, v in st.items()}
        st["R"], st["k"] = self.R, self.k
        st["field"] = self.field.snapshot(host)
        return st

    def restore(self, st):
        """Resumes from a ``snapshot`` (device or host arrays)."""
        cur = self.cur
        self.W[cur].copy_(torch.as_tensor(st["W"]))
        self.wg[cur].copy_(torch.as_tensor(st["wg"]))
        self.wa[cur].copy_(torch.as_tensor(st["wa"]))
        self.gamma.copy_(torch.as_tensor(st["gamma"]))
        self.gamma_prev.copy_(torch.as_tensor(st["gamma_prev"]))
        self.R, self.k = int(st["R"]), int(st["k"])
        if self._cl.numel() < self.k:
            grow = self.k - self._cl.numel() + 4096
            self._cl = torch.cat([self._cl, torch.zeros(grow, dtype=self._cl.dtype,
                                                        device=self.device)])
            self._cdi = torch.cat([self._cdi, torch.zeros(grow, dtype=self._cdi.dtype,
                                                          device=self.device)])
        self._cl[: self.k].copy_(torch.as_tensor(st["cl"]))
        self._cdi[: self.k].copy_(torch.as_tensor(st["cdi"]))
        self.field.restore(st["field"])

    def _rc0_bound(self):
        if not hasattr(self, "_rcb"):
            self._rcb = torch.full((self.P,), self.cfg.rc0, dtype=torch.float64,
                                   device=self.device)
        return self._rcb

    @property
    def cl(self):
        return self._cl[: self.k].cpu().numpy()

    @property
    def cdi(self):
        return self._cdi[: self.k].cpu().numpy()
