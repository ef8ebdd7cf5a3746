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
from fluxvortex_gb300.geometry import Lattice, lattice
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


def reference_panels(cfg, base, L0, w_nodes, th_nodes, y_nodes):
    """The reference's panel deformation (aeroelastic_solver.py:150-221): every
    panel moves with the beam's heave w and twist theta interpolated at its own
    collocation span station |y_c| (no shared vertices: neighbouring panels
    move apart at their common edges).  Each of its corners and ring-vortex
    vertices moves by dz = w - (x - x_ea) sin(theta), dx = (x - x_ea)
    (cos(theta) - 1) (theta nose-up here; the reference counts it nose-down,
    dz = w + (x - x_ea) sin(theta_ref)); the collocation point by dz only.
    Normals and areas follow from the moved corners.  The wake's first vertex
    row is the back row of the last chordwise panels' rings (strip j's
    back-left vertex, the last strip's back-right vertex)."""
    nc, ns = cfg.nc, cfg.ns
    x_ea = cfg.x_ea * cfg.chord
    yc = np.abs(L0.colloc[:, 1])
    w = np.interp(yc, y_nodes, w_nodes)
    th = np.interp(yc, y_nodes, th_nodes)
    s, c1 = np.sin(th)[:, None], (np.cos(th) - 1.0)[:, None]

    def move(p):
        xr = p[:, 0:1] - x_ea
        out = p.copy()
        out[:, 0:1] += xr * c1
        out[:, 2:3] += w[:, None] - xr * s
        return out

    i, j = np.divmod(np.arange(nc * ns), ns)
    c00, c01 = move(base[i, j]), move(base[i, j + 1])
    c10, c11 = move(base[i + 1, j]), move(base[i + 1, j + 1])
    cr = np.cross(c11 - c00, c01 - c10)
    nrm = np.linalg.norm(cr, axis=1)
    br, fr, fl, bl = move(L0.br), move(L0.fr), move(L0.fl), move(L0.bl)
    colloc = L0.colloc.copy()
    colloc[:, 2] += w - (colloc[:, 0] - x_ea) * np.sin(th)
    last = np.arange((nc - 1) * ns, nc * ns)
    te = np.vstack([bl[last], br[last[-1]][None]])
    return Lattice(br=br, fr=fr, fl=fl, bl=bl, colloc=colloc, normal=cr / nrm[:, None],
                   area=0.5 * nrm, leg_center=0.5 * (fr + fl), leg_vec=fl - fr, te_back=te,
                   nc=nc, ns=ns)


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
        self.reference = cfg.coupling == "reference"
        if self.reference:
            # the reference couples from step 1 on and applies each coupling's
            # deformation to the next step's geometry: steps 0 and 1 run on
            # the undeformed wing (aeroelastic_solver.py:63-66, :108-110)
            self.L0 = lattice(self.base)
            self.geom_d = np.zeros_like(self.beam.d)
            self.n_total = cfg.n_steps(V)
            self.W = self._ref_lattice(self.geom_d).te_back[None].copy()
        else:
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

    def _ref_lattice(self, d):
        b = self.beam
        return reference_panels(self.cfg, self.base, self.L0, d[0::3], d[2::3], b.y_nodes)

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
        if self.reference:
            # vertices mutated only: no motion velocity in the boundary
            # condition or the loads
            L = self._ref_lattice(self.geom_d)
            v_col = v_leg = np.zeros((L.colloc.shape[0], 3))
        else:
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
        y_st = (np.arange(L.ns) + 0.5) * cfg.semi_span / L.ns
        if self.reference:
            # station lift and its moment about x = 0 with the collocation
            # point's chordwise position x_c as the arm (aeroelastic_solver.py:
            # 126-138: lift -F_z in PteraSoftware's axes, moment x_c (-F_z)
            # nose-down); here lift F_z and the nose-up moment -x_c F_z.
            # Coupling from step 1 to the step before the last (:63-71); the
            # next step's geometry from the new displacements
            lift = Fz.sum(axis=0)
            torque = (-self.L0.colloc[:, 0].reshape(L.nc, L.ns) * Fz).sum(axis=0)
            if 1 <= self.k < self.n_total - 1:
                self.beam.step(distribute(self.beam.y_nodes, y_st, lift, torque), cfg.dt)
                self.tip_w.append(self.beam.d[-3])
                self.tip_theta.append(self.beam.d[-1])
                self.geom_d = self.beam.d.copy()
            te = self._ref_lattice(self.geom_d).te_back
        else:
            x_ea = cfg.x_ea * cfg.chord
            arm = x_ea - L.leg_center[:, 0].reshape(L.nc, L.ns)
            lift = Fz.sum(axis=0)
            torque = (Fz * arm).sum(axis=0)
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
