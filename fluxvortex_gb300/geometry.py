"""Wing lattices and kinematics for the PteraSoftware-free hybrid step.

PteraSoftware, which builds the reference's geometries, is a third-party
package that is not available; this module builds the same kinds of wings
from their definitions (NACA 4-digit mean lines, uniform / cosine spacing,
mirror symmetry) in the axes PteraSoftware uses for its panels: x aft, y to
the right (span), z up.

A wing is a vertex grid ``verts[nc+1, ns+1, 3]`` (chordwise rows LE -> TE,
spanwise columns left -> right).  Ring vortices sit on the quarter-chord
lattice (each ring's front leg on its panel's quarter chord, the last row's
back leg a quarter panel behind the trailing edge), collocation points at the
three-quarter chord, as in a standard ring-vortex UVLM (Katz & Plotkin ch.
13; the reference's PS-free lattice in newton_pc/adapters/flap.py:327-336 uses
the same offsets).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


def naca4_camber(x, m, p):
    """Mean line z/c of a NACA mpXX section at x/c (m, p as fractions)."""
    x = np.asarray(x, dtype=np.float64)
    if m == 0.0 or p == 0.0:
        return np.zeros_like(x)
    return np.where(x < p, m / p ** 2 * (2 * p * x - x ** 2),
                    m / (1 - p) ** 2 * ((1 - 2 * p) + 2 * p * x - x ** 2))


def spacing(n, kind):
    """n+1 stations on [0, 1]: 'uniform' or 'cosine' (clustered at both ends)."""
    s = np.linspace(0.0, 1.0, n + 1)
    if kind == "cosine":
        return 0.5 * (1.0 - np.cos(np.pi * s))
    return s


def rectangular_wing(chord, semi_span, nc, ns, camber=(0.0, 0.0), span_spacing="uniform",
                     symmetric=True, root_chord=None, tip_chord=None, y0=0.0):
    """Vertex grid of a (tapered) wing; with ``symmetric`` the half wing of ns
    panels is mirrored about y = y0, giving 2 ns spanwise panels."""
    cr = chord if root_chord is None else root_chord
    ct = chord if tip_chord is None else tip_chord
    xs = spacing(nc, "uniform")
    ys = spacing(ns, span_spacing) * semi_span
    m, p = camber
    zc = naca4_camber(xs, m, p)
    verts = np.zeros((nc + 1, ns + 1, 3))
    for j, y in enumerate(ys):
        c = cr + (ct - cr) * (y / semi_span)
        verts[:, j, 0] = xs * c
        verts[:, j, 1] = y0 + y
        verts[:, j, 2] = zc * c
    if symmetric:
        left = verts[:, ::-1, :].copy()
        left[:, :, 1] = 2 * y0 - left[:, :, 1]
        verts = np.concatenate([left[:, :-1, :], verts], axis=1)
    return verts


@dataclass
class Lattice:
    """Ring-vortex lattice of one vertex grid (all arrays (P, 3) or (P,))."""
    br: np.ndarray
    fr: np.ndarray
    fl: np.ndarray
    bl: np.ndarray
    colloc: np.ndarray
    normal: np.ndarray
    area: np.ndarray
    leg_center: np.ndarray   # centre of each ring's front (bound) leg
    leg_vec: np.ndarray      # FR -> FL of each ring's front leg
    te_back: np.ndarray      # (ns+1, 3) back edge of the trailing-edge rings
    nc: int
    ns: int


def lattice(verts) -> Lattice:
    nc, ns = verts.shape[0] - 1, verts.shape[1] - 1
    vq = np.empty_like(verts)
    vq[:-1] = verts[:-1] + 0.25 * (verts[1:] - verts[:-1])
    vq[-1] = verts[-1] + 0.25 * (verts[-1] - verts[-2])
    fl = vq[:-1, :-1].reshape(-1, 3)
    fr = vq[:-1, 1:].reshape(-1, 3)
    br = vq[1:, 1:].reshape(-1, 3)
    bl = vq[1:, :-1].reshape(-1, 3)
    vc = verts[:-1] + 0.75 * (verts[1:] - verts[:-1])
    colloc = (0.5 * (vc[:, :-1] + vc[:, 1:])).reshape(-1, 3)
    d1 = (verts[1:, 1:] - verts[:-1, :-1]).reshape(-1, 3)
    d2 = (verts[:-1, 1:] - verts[1:, :-1]).reshape(-1, 3)
    cr = np.cross(d1, d2)
    nrm = np.linalg.norm(cr, axis=1)
    return Lattice(br=np.ascontiguousarray(br), fr=np.ascontiguousarray(fr),
                   fl=np.ascontiguousarray(fl), bl=np.ascontiguousarray(bl),
                   colloc=np.ascontiguousarray(colloc), normal=cr / nrm[:, None],
                   area=0.5 * nrm, leg_center=0.5 * (fr + fl), leg_vec=fl - fr,
                   te_back=vq[-1].copy(), nc=nc, ns=ns)


@dataclass
class Kinematics:
    """Rigid motion of the wing: heave z(t) = h0 sin(2 pi t / T + phase) and a
    flapping rotation about the x axis through y = y0, theta(t) = A sin(2 pi t / T)
    applied to |y - y0| (both half wings rotate up together)."""
    heave_amp: float = 0.0
    flap_amp: float = 0.0          # radians
    period: float = 1.0
    y0: float = 0.0

    def vertices(self, base, t):
        v = base.copy()
        w = 2.0 * np.pi / self.period
        if self.flap_amp:
            th = self.flap_amp * np.sin(w * t)
            dy = v[..., 1] - self.y0
            s = np.sign(dy)
            y, z = np.abs(dy), v[..., 2]
            v[..., 1] = self.y0 + s * (y * np.cos(th) - z * np.sin(th))
            v[..., 2] = y * np.sin(th) + z * np.cos(th)
        if self.heave_amp:
            v[..., 2] += self.heave_amp * np.sin(w * t)
        return v

    def rates(self, t):
        """(heave, heave rate, flap-angle rate) at time t."""
        w = 2.0 * np.pi / self.period
        return (self.heave_amp * np.sin(w * t), self.heave_amp * w * np.cos(w * t),
                self.flap_amp * w * np.cos(w * t))

    def point_velocity(self, p, t):
        """Velocity of body points at current positions p (P,3): heave rate on
        z plus the flapping rotation about the x axis through y0, mirrored for
        the left half (v = s thetadot (0, -Z, dY), s = sign(dY))."""
        h, hdot, thdot = self.rates(t)
        p = np.asarray(p, dtype=np.float64)
        v = np.zeros_like(p)
        dy = p[:, 1] - self.y0
        s = np.where(dy >= 0.0, 1.0, -1.0)
        Z = p[:, 2] - h
        v[:, 1] = -s * thdot * Z
        v[:, 2] = s * thdot * dy + hdot
        return v


@dataclass
class HybridConfig:
    """One hybrid panel-particle case (BASELINE configs 1, 2, 5 shapes)."""
    verts: np.ndarray
    u_inf: np.ndarray
    dt: float
    kin: Kinematics = field(default_factory=Kinematics)
    rho: float = 1.225
    rc0: float = 0.03
    nu: float = 0.0
    n_keep: int = 10
    sigma_rule: str = "v_dt"       # 'v_dt' (HybridSolver :157) or 'edge' (1.3 x mean edge)
    free_vpm: bool = True
    stretch: bool = False
    # Pedrizzetti relaxation is off by default for the panel-particle configs:
    # the reference's value (0.3) acts through the rounding noise of its
    # Gaussian-erf self-pair term; with the analytic self term it destabilises
    # the converted ring-leg wake.
    rlxf: float = 0.0
    kernel: str = "winckelmans"
    max_particles: int = 200000
    far_field: str = None          # None: direct self-sweeps; "tree": treecode

    @property
    def speed(self):
        return float(np.linalg.norm(self.u_inf))


def heaving_wing(n_keep=10, steps_per_cycle=40, k=0.5, h0c=0.1, V=10.0, chord=1.0,
                 half_span=5.0, nc=10, ns=6, **kw) -> HybridConfig:
    """The heaving NACA 0012 wing: chord 1, half span 5 (mirrored), nc=10 x ns=6
    per half, V = 10 m/s, h0/c = 0.1 at reduced frequency k (k = omega c / 2V)."""
    omega = 2 * k * V / chord
    period = 2 * np.pi / omega
    verts = rectangular_wing(chord, half_span, nc, ns)
    return HybridConfig(verts=verts, u_inf=np.array([V, 0.0, 0.0]), dt=period / steps_per_cycle,
                        kin=Kinematics(heave_amp=h0c * chord, period=period), rc0=0.03 * chord,
                        n_keep=n_keep, **kw)


def static_wing(alpha_deg=5.0, V=10.0, chord=2.0, semi_span=5.0, nc=7, ns=18, n_keep=1000,
                **kw) -> HybridConfig:
    """The static NACA 2412 wing: chord 2, semi-span 5, nc=7 x ns=18 cosine,
    dt = panel chord / V."""
    verts = rectangular_wing(chord, semi_span, nc, ns, camber=(0.02, 0.4), span_spacing="cosine",
                             symmetric=False)
    a = np.radians(alpha_deg)
    return HybridConfig(verts=verts, u_inf=V * np.array([np.cos(a), 0.0, np.sin(a)]),
                        dt=chord / nc / V, rc0=0.03 * chord, n_keep=n_keep, **kw)
