"""CPU oracle of one flutter-sweep environment (TEST INFRASTRUCTURE ONLY).

FP64 NumPy restatement of the coupled UVLM + beam time history that the
flutter-sweep kernel runs per airspeed.  The reference's coupling loop is
AeroelasticSolver._structural_coupling / _deform_panels
(src/fluxvortex/aeroelastic_solver.py:68-221) around PteraSoftware's solver
(absent here); the model's deviations from it are listed in
fluxvortex_gb300/flutter.py.  Per step:
  1. deformed vertices and their velocities from the beam state;
  2. AIC (expanded ring Biot-Savart . n), wake rings + particles at the
     collocation points, rhs = -((U - v_body) + V_wake) . n, FP64 solve;
  3. Kutta-Joukowski loads on the bound legs with the full induced velocity
     minus rho dGamma/dt A n (as oracle/hybrid.py);
  4. station lift / torque -> nodal loads (oracle.beam.distribute), Newmark
     step (oracle.beam.Beam, restating beam_fe.py);
  5. shed the trailing-edge row at the next geometry, convect the ring rows
     and the particles with the freestream, convert rows >= n_keep to
     particles (experiment_hybrid_panel_particle.py:145-204 with sigma =
     1.3 x mean edge), keep the newest max_particles.
Biot-Savart evaluations go through ``oracle.oracle`` (pinned to the
reference's golden vectors); the beam through ``oracle.beam`` (pinned to the
reference's BeamFE).
"""
from __future__ import annotations

import math

import numpy as np

from fluxvortex_gb300.flutter import FlutterConfig
from fluxvortex_gb300.geometry import lattice
from oracle import oracle as O
from oracle.beam import Beam, distribute


def lattice_point_velocities(vel):
    """Velocities of the collocation points and bound-leg centres: the same
    linear combinations of the vertex velocities as the points of the vertices."""
    vq = np.empty_like(vel)
    vq[:-1] = vel[:-1] + 0.25 * (vel[1:] - vel[:-1])
    vq[-1] = vel[-1] + 0.25 * (vel[-1] - vel[-2])
    vc = vel[:-1] + 0.75 * (vel[1:] - vel[:-1])
    col = (0.5 * (vc[:, :-1] + vc[:, 1:])).reshape(-1, 3)
    leg = (0.5 * (vq[:-1, :-1] + vq[:-1, 1:])).reshape(-1, 3)
    return col, leg


class FlutterOracle:
    def __init__(self, cfg: FlutterConfig, V):
        self.cfg = cfg
        self.V = float(V)
        self.u_inf = cfg.u_inf(V)
        self.base = cfg.base_vertices()
        self.beam = Beam(**cfg.beam)
        tip = self.beam.nnodes - 1
        self.beam.d[3 * tip] = cfg.tip_w
        self.beam.d[3 * tip + 2] = math.radians(cfg.tip_theta_deg)
        self.beam.init_acceleration()
        self.ns = cfg.ns
        verts, _ = self.deform()
        self.W = lattice(verts).te_back[None].copy()
        self.wgam = np.zeros((0, cfg.ns))
        self.wage = np.zeros(0)
        self.p_pos = np.zeros((0, 3))
        self.p_alp = np.zeros((0, 3))
        self.p_sig = np.zeros(0)
        self.gamma_prev = None
        self.tip_w, self.tip_theta = [], []
        self.k = 0

    def deform(self):
        cfg, b = self.cfg, self.beam
        y = self.base[..., 1]
        w = np.interp(y, b.y_nodes, b.d[0::3])
        th = np.interp(y, b.y_nodes, b.d[2::3])
        wd = np.interp(y, b.y_nodes, b.v[0::3])
        thd = np.interp(y, b.y_nodes, b.v[2::3])
        x_ea = cfg.x_ea * cfg.chord
        xr = self.base[..., 0] - x_ea
        verts = self.base.copy()
        verts[..., 0] = x_ea + xr * np.cos(th)
        verts[..., 2] = self.base[..., 2] + w - xr * np.sin(th)
        vel = np.zeros_like(verts)
        vel[..., 0] = -xr * np.sin(th) * thd
        vel[..., 2] = wd - xr * np.cos(th) * thd
        return verts, vel

    def _rings(self):
        W, R, ns = self.W, self.wgam.shape[0], self.ns
        if R == 0:
            e = np.zeros((0, 3))
            return e, e, e, e, np.zeros(0), np.zeros(0), np.zeros(0)
        fl = W[:R, :-1].reshape(-1, 3)
        fr = W[:R, 1:].reshape(-1, 3)
        br = W[1:R + 1, 1:].reshape(-1, 3)
        bl = W[1:R + 1, :-1].reshape(-1, 3)
        return (br, fr, fl, bl, self.wgam.reshape(-1), np.full(R * ns, self.cfg.rc0),
                np.repeat(self.wage, ns))

    def _induced(self, pts, rings):
        br, fr, fl, bl, g, rc, ages = rings
        v = O.collapsed_velocities_from_ring_vortices(pts, br, fr, fl, bl, g, rc, None, ages,
                                                      self.cfg.nu)
        if self.p_pos.shape[0]:
            v = v + O.velocity_from_particles(pts, self.p_pos, self.p_alp, self.p_sig,
                                              "winckelmans")
        return v

    def step(self):
        cfg = self.cfg
        verts, vel = self.deform()
        L = lattice(verts)
        v_col, v_leg = lattice_point_velocities(vel)
        P = L.colloc.shape[0]
        rc_b = np.full(P, cfg.rc0)
        E = O.expanded_velocities_from_ring_vortices(L.colloc, L.br, L.fr, L.fl, L.bl,
                                                     np.ones(P), rc_b, None, None, cfg.nu)
        A = np.einsum("ijc,ic->ij", E, L.normal)
        rings = self._rings()
        Vw = self._induced(L.colloc, rings)
        rhs = -np.einsum("ic,ic->i", (self.u_inf[None, :] - v_col) + Vw, L.normal)
        gam = np.linalg.solve(A, rhs)
        Vl = self._induced(L.leg_center, rings)
        Vb = O.collapsed_velocities_from_ring_vortices(L.leg_center, L.br, L.fr, L.fl, L.bl, gam,
                                                       rc_b, None, None, cfg.nu)
        V = (self.u_inf[None, :] - v_leg) + Vl + Vb
        g2 = gam.reshape(L.nc, L.ns)
        geff = g2.copy()
        geff[1:] -= g2[:-1]
        gprev = gam if self.gamma_prev is None else self.gamma_prev
        dgdt = (gam - gprev) / cfg.dt
        F = (cfg.rho * geff.reshape(-1)[:, None] * np.cross(V, L.leg_vec)
             - (cfg.rho * dgdt * L.area)[:, None] * L.normal)
        Fz = F[:, 2].reshape(L.nc, L.ns)
        x_ea = cfg.x_ea * cfg.chord
        arm = x_ea - L.leg_center[:, 0].reshape(L.nc, L.ns)
        lift = Fz.sum(axis=0)
        torque = (Fz * arm).sum(axis=0)
        y_st = (np.arange(L.ns) + 0.5) * cfg.semi_span / L.ns
        self.beam.step(distribute(self.beam.y_nodes, y_st, lift, torque), cfg.dt)
        self.tip_w.append(self.beam.d[-3])
        self.tip_theta.append(self.beam.d[-1])
        # wake: convect, shed at the next geometry, convert old rows
        verts_n, _ = self.deform()
        te = lattice(verts_n).te_back
        if self.p_pos.shape[0]:
            self.p_pos = self.p_pos + self.u_inf * cfg.dt
        self.W = np.concatenate([te[None], self.W + self.u_inf * cfg.dt], axis=0)
        self.wgam = np.concatenate([g2[-1][None], self.wgam], axis=0)
        self.wage = np.concatenate([[0.0], self.wage + cfg.dt])
        R = self.wgam.shape[0]
        if R > cfg.n_keep:
            pos, alp, sig = [], [], []
            for r in range(cfg.n_keep, R):
                for j in range(self.ns):
                    g = self.wgam[r, j]
                    if abs(g) < 1e-15:
                        continue
                    fl, fr = self.W[r, j], self.W[r, j + 1]
                    bl, br = self.W[r + 1, j], self.W[r + 1, j + 1]
                    s = 1.3 * 0.25 * (np.linalg.norm(fl - fr) + np.linalg.norm(bl - fl)
                                      + np.linalg.norm(br - bl) + np.linalg.norm(fr - br))
                    for a, b in ((fr, fl), (fl, bl), (bl, br), (br, fr)):
                        al = g * (b - a)
                        if al @ al > 1e-30:
                            pos.append(0.5 * (a + b))
                            alp.append(al)
                            sig.append(s)
            if pos:
                self.p_pos = np.vstack([self.p_pos, pos])
                self.p_alp = np.vstack([self.p_alp, alp])
                self.p_sig = np.concatenate([self.p_sig, sig])
            self.W = self.W[:cfg.n_keep + 1]
            self.wgam = self.wgam[:cfg.n_keep]
            self.wage = self.wage[:cfg.n_keep]
        excess = self.p_pos.shape[0] - cfg.max_particles
        if excess > 0:
            self.p_pos = self.p_pos[excess:]
            self.p_alp = self.p_alp[excess:]
            self.p_sig = self.p_sig[excess:]
        self.gamma_prev = gam
        self.k += 1
        return gam

    def run(self, n_steps=None):
        n = self.cfg.n_steps(self.V) if n_steps is None else n_steps
        for _ in range(n):
            self.step()
        return np.array(self.tip_w), np.array(self.tip_theta)
