"""CPU oracle of the hybrid panel-particle step (TEST INFRASTRUCTURE ONLY).

A NumPy restatement, in FP64, of one step of the reference's hybrid solver
(tests/experiment_hybrid_panel_particle.py:87-204 of the FLUXVortex project)
on a PteraSoftware-free ring-vortex UVLM.  PteraSoftware's solver loop is a
third-party dependency that is absent; its per-step order, as the reference
documents it (idea-stage/architecture_analysis.md:7-27) and as HybridSolver
overrides it, is followed:

  1. wing-wing influences: AIC[i,j] = (unit ring j at collocation i) . n_i
     -> expanded_velocities_from_ring_vortices (warp_kernels.py:305-332)
  2. freestream + body motion, 3. wake-wing influences: ring rows kept as
     panels -> collapsed_velocities_from_ring_vortices (warp_kernels.py:251)
     plus the vortex particles -> velocity_from_particles
     (experiment_hybrid_panel_particle.py:114-123)
  4. strengths: AIC Gamma = -(U_inf - v_body + V_wake) . n (FP64 solve)
  5. loads (``loads="bernoulli"``: the unsteady Bernoulli pressure of
     newton_pc/adapters/flap.py:357-377 instead): Kutta-Joukowski on each
     ring's bound (front) leg, F = rho
     (Gamma_ij - Gamma_i-1,j) (V x l), with V the freestream minus the body
     motion plus the velocity induced by every bound ring, the wake rings and
     the particles (segments collinear with the leg are skipped by the
     kernel's own tests, warp_kernels.py:81), plus the unsteady term
     -rho dGamma/dt A n
  6. populate the next wake: convect the ring-wake lattice with the
     freestream (prescribed wake) or, with ``free_ring_wake``, each vertex with
     the freestream plus the velocity the bound rings, wake rings and particles
     induce at it (PteraSoftware's free wake), attach a new row whose strength
     is the trailing-edge ring's, ages += dt
  7. HybridSolver._convert_old_wake_to_particles (:145-204): rows >= N_keep
     become 4 particles per ring (leg midpoints, alpha = Gamma (b - a)),
     rings with |Gamma| < 1e-15 and legs with |alpha|^2 <= 1e-30 skipped
  8. particle convection: VortexParticleField.advect_rk3 (particles.py:85)
     with U_inf and free-wake self-induction (:125-143), then relaxation.

Several lifting surfaces (PteraSoftware's multi-wing airplanes, e.g.
tests/benchmark_flapping.py:28-141) share one vertex grid: strip j spans
vertex columns col[j], col[j]+1, each surface sheds its own wake strips from
its own trailing-edge vertices, and each moves with its own kinematics.

Every Biot-Savart evaluation goes through ``oracle.oracle`` (the C
restatement pinned to the reference's golden vectors).
"""
from __future__ import annotations

import numpy as np

from fluxvortex_gb300.geometry import HybridConfig, lattice
from oracle import oracle as O
from oracle import population as POP


class HybridOracle:
    def __init__(self, cfg: HybridConfig):
        self.cfg = cfg
        self.k = 0
        self.col = cfg.layout()[0]
        ns = self.col.size
        self.ns = ns
        L0 = lattice(cfg.vertices(0.0), self.col)
        self.W = L0.te_back[None].copy()        # wake vertex rows, newest first
        self.wgam = np.zeros((0, ns))
        self.wage = np.zeros(0)
        self.p_pos = np.zeros((0, 3))
        self.p_gam = np.zeros((0, 3))
        self.p_sig = np.zeros(0)
        self.p_age = np.zeros(0)
        self.gamma_prev = None
        self.cl, self.cdi = [], []
        self.gamma = None
        self.n_merged = 0

    # ring wake in the five-function layout
    def wake_rings(self):
        W, R, ns = self.W, self.wgam.shape[0], self.ns
        if R == 0:
            e = np.zeros((0, 3))
            return e, e, e, e, np.zeros(0), np.zeros(0), np.zeros(0)
        a, b = self.col, self.col + 1
        fl = W[:R, a].reshape(-1, 3)
        fr = W[:R, b].reshape(-1, 3)
        br = W[1:R + 1, b].reshape(-1, 3)
        bl = W[1:R + 1, a].reshape(-1, 3)
        g = self.wgam.reshape(-1)
        rc = np.full(R * ns, self.cfg.rc0)
        ages = np.repeat(self.wage, ns)
        return br, fr, fl, bl, g, rc, ages

    def _induced(self, pts, rings):
        """Wake rings + particles at pts."""
        br, fr, fl, bl, g, rc, ages = rings
        v = O.collapsed_velocities_from_ring_vortices(pts, br, fr, fl, bl, g, rc, None, ages,
                                                      self.cfg.nu)
        if self.p_pos.shape[0]:
            v = v + O.velocity_from_particles(pts, self.p_pos, self.p_gam, self.p_sig,
                                              self.cfg.kernel)
        return v

    def _bernoulli(self, verts, L, gam, Vext, t):
        """Unsteady Bernoulli loads (newton_pc/adapters/flap.py:357-377) on this
        lattice: tangents between vertex-edge midpoints, circulation gradients
        restarting at the first row and each surface's first strip,
        dp = rho (V . t_c dG/dc + V . t_s dG/ds + dG/dt), F = sum dp A n."""
        cfg = self.cfg
        nc, ns = L.nc, L.ns
        a, b = self.col, self.col + 1
        v0, v1 = verts[:-1], verts[1:]
        tau_c = (0.5 * (v1[:, b] + v1[:, a]) - 0.5 * (v0[:, b] + v0[:, a])).reshape(-1, 3)
        tau_s = (0.5 * (v1[:, b] + v0[:, b]) - 0.5 * (v1[:, a] + v0[:, a])).reshape(-1, 3)
        dc = np.linalg.norm(tau_c, axis=1)
        ds = np.linalg.norm(tau_s, axis=1)
        g2 = gam.reshape(nc, ns)
        gc = g2.copy()
        gc[1:] -= g2[:-1]
        first = np.r_[True, self.col[1:] != self.col[:-1] + 1]
        gs = g2.copy()
        gs[:, ~first] -= g2[:, np.flatnonzero(~first) - 1]
        vb = cfg.point_velocity(L.colloc, t)
        V = (cfg.u_inf[None, :] - vb) + Vext
        gprev = gam if self.gamma_prev is None else self.gamma_prev
        # flap.py's rings circulate opposite to PteraSoftware's (these
        # strengths, flap.py:330-332): the same flow gives -dp here
        dp = -cfg.rho * (np.einsum("ic,ic->i", V, tau_c) / dc * (gc.reshape(-1) / dc)
                         + np.einsum("ic,ic->i", V, tau_s) / ds * (gs.reshape(-1) / ds)
                         + (gam - gprev) / cfg.dt)
        Ft = (dp * L.area)[:, None] * L.normal
        Ft = Ft.sum(axis=0)
        V0 = cfg.speed
        eD = cfg.u_inf / V0
        eL = np.array([-eD[2], 0.0, eD[0]])
        qS = 0.5 * cfg.rho * V0 ** 2 * (L.area.sum() if cfg.s_ref is None else cfg.s_ref)
        self.cl.append(float(Ft @ eL / qS))
        self.cdi.append(float(Ft @ eD / qS))

    def step(self):
        cfg = self.cfg
        t = self.k * cfg.dt
        verts = cfg.vertices(t)
        L = lattice(verts, self.col)
        P = L.colloc.shape[0]
        ones = np.ones(P)
        rc_b = np.full(P, cfg.rc0)
        # 1. AIC
        E = O.expanded_velocities_from_ring_vortices(L.colloc, L.br, L.fr, L.fl, L.bl, ones, rc_b,
                                                     None, None, cfg.nu)
        A = np.einsum("ijc,ic->ij", E, L.normal)
        # 2-3. freestream, body motion, wake
        rings = self.wake_rings()
        Vw = self._induced(L.colloc, rings)
        vb = cfg.point_velocity(L.colloc, t)
        rhs = -np.einsum("ic,ic->i", (cfg.u_inf[None, :] - vb) + Vw, L.normal)
        # 4. strengths
        gam = np.linalg.solve(A, rhs)
        # 5. loads
        if cfg.loads == "bernoulli":
            self._bernoulli(verts, L, gam, Vw, t)
            Vl = None
        else:
            Vl = self._induced(L.leg_center, rings)
        if Vl is not None:
            Vb = O.collapsed_velocities_from_ring_vortices(L.leg_center, L.br, L.fr, L.fl, L.bl, gam,
                                                           rc_b, None, None, cfg.nu)
            vbl = cfg.point_velocity(L.leg_center, t)
            V = (cfg.u_inf[None, :] - vbl) + (Vl + Vb)
            g2 = gam.reshape(L.nc, L.ns)
            geff = g2.copy()
            geff[1:] -= g2[:-1]
            gprev = gam if self.gamma_prev is None else self.gamma_prev
            dgdt = (gam - gprev) / cfg.dt
            F = (cfg.rho * geff.reshape(-1)[:, None] * np.cross(V, L.leg_vec)
                 - (cfg.rho * dgdt * L.area)[:, None] * L.normal)
            Ft = F.sum(axis=0)
            V0 = cfg.speed
            eD = cfg.u_inf / V0
            eL = np.array([-eD[2], 0.0, eD[0]])
            qS = 0.5 * cfg.rho * V0 ** 2 * (L.area.sum() if cfg.s_ref is None else cfg.s_ref)
            self.cl.append(float(Ft @ eL / qS))
            self.cdi.append(float(Ft @ eD / qS))
        # 6. next wake
        g2 = gam.reshape(L.nc, L.ns)
        Ln = lattice(cfg.vertices(t + cfg.dt), self.col)
        if cfg.free_ring_wake:
            # free ring wake: each old vertex moves with u_inf + bound rings +
            # wake rings + particles at it
            pts = self.W.reshape(-1, 3)
            rc_b = np.full(L.colloc.shape[0], cfg.rc0)
            V = cfg.u_inf[None, :] + O.collapsed_velocities_from_ring_vortices(
                pts, L.br, L.fr, L.fl, L.bl, gam, rc_b, None, None, cfg.nu)
            if rings[4].size:
                br, fr, fl, bl, g, rc, ages = rings
                V = V + O.collapsed_velocities_from_ring_vortices(pts, br, fr, fl, bl, g, rc, None,
                                                                  ages, cfg.nu)
            if self.p_pos.shape[0]:
                V = V + O.velocity_from_particles(pts, self.p_pos, self.p_gam, self.p_sig,
                                                  cfg.kernel)
            Wc = self.W + V.reshape(self.W.shape) * cfg.dt
        else:
            Wc = self.W + cfg.u_inf * cfg.dt
        self.W = np.concatenate([Ln.te_back[None], Wc], axis=0)
        self.wgam = np.concatenate([g2[-1][None], self.wgam], axis=0)
        self.wage = np.concatenate([[0.0], self.wage + cfg.dt])
        # 7. rows >= N_keep -> particles
        R = self.wgam.shape[0]
        if R > cfg.n_keep:
            pos, alp, sig = [], [], []
            for r in range(cfg.n_keep, R):
                for j in range(self.ns):
                    g = self.wgam[r, j]
                    if abs(g) < 1e-15:
                        continue
                    c = self.col[j]
                    fl, fr = self.W[r, c], self.W[r, c + 1]
                    bl, br = self.W[r + 1, c], self.W[r + 1, c + 1]
                    if cfg.sigma_rule == "edge":
                        s = 1.3 * 0.25 * (np.linalg.norm(fl - fr) + np.linalg.norm(bl - fl)
                                          + np.linalg.norm(br - bl) + np.linalg.norm(fr - br))
                    else:
                        s = cfg.speed * cfg.dt
                    for a, b in ((fr, fl), (fl, bl), (bl, br), (br, fr)):
                        al = g * (b - a)
                        if al @ al > 1e-30:
                            pos.append(0.5 * (a + b))
                            alp.append(al)
                            sig.append(s)
            if pos:
                self.p_pos = np.vstack([self.p_pos, pos])
                self.p_gam = np.vstack([self.p_gam, alp])
                self.p_sig = np.concatenate([self.p_sig, sig])
                self.p_age = np.concatenate([self.p_age, np.zeros(len(pos))])
            self.W = self.W[:cfg.n_keep + 1]
            self.wgam = self.wgam[:cfg.n_keep]
            self.wage = self.wage[:cfg.n_keep]
        # 8. particles
        if self.p_pos.shape[0]:
            self.p_pos, self.p_gam, self.p_sig, self.p_age = O.advect_rk3(
                self.p_pos, self.p_gam, self.p_sig, self.p_age, cfg.dt, cfg.u_inf, cfg.kernel,
                cfg.nu, cfg.rlxf, cfg.stretch, cfg.free_vpm)
        # 9. population control (newton_pc/adapters/flap.py:469-475)
        state = (self.p_pos, self.p_gam, self.p_sig, self.p_age)
        if cfg.population == "drop":
            state = POP.drop_oldest(*state, cfg.pop_max)
        elif cfg.population == "merge" and self.p_pos.shape[0]:
            *state, merged = POP.merge_pass(*state, cfg.ref_points(L.colloc), cfg.speed,
                                            cfg.merge_eps, cfg.merge_protect,
                                            cfg.merge_protect_dist)
            self.n_merged += merged
        self.p_pos, self.p_gam, self.p_sig, self.p_age = state
        self.gamma_prev = gam
        self.gamma = gam
        self.k += 1
        return self.cl[-1], self.cdi[-1]
