"""Wing lattices and kinematics for the PteraSoftware-free hybrid step.

PteraSoftware, which builds the reference's geometries, is a third-party
package that is not available; this module builds the same kinds of wings
from their definitions (NACA 4-digit mean lines, uniform / cosine spacing,
mirror symmetry) in the axes PteraSoftware uses for its panels: x aft, y to
the right (span), z up.

A wing is a vertex grid ``verts[nc+1, ns+1, 3]`` (chordwise rows LE -> TE,
spanwise columns left -> right).  Several lifting surfaces with the same
chordwise count share one grid whose columns are the surfaces' spanwise
stations side by side (``combine``): ring strip j spans vertex columns
``col[j]`` and ``col[j] + 1`` and vertex column c moves with surface
``surf[c]``; one surface is ``col = 0..ns-1``, ``surf = 0``.  Ring vortices sit on the quarter-chord
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


def _rot_y(deg):
    a = np.radians(deg)
    c, s = np.cos(a), np.sin(a)
    return np.array([[c, 0.0, s], [0.0, 1.0, 0.0], [-s, 0.0, c]])


def lofted_wing(sections, nc, ns, span_spacing="uniform", camber=(0.0, 0.0), origin=(0, 0, 0),
                incidence=0.0):
    """Vertex grid (nc+1, ns+1, 3) of one wing panel between two cross
    sections, PteraSoftware style: each section is (leading point, chord,
    twist in degrees about y through its leading point; positive = trailing
    edge down); the section mean lines are sampled at nc+1 uniform chord
    stations and the spanwise vertices interpolate linearly between the two
    sections at ``span_spacing`` stations.  The whole wing is then pitched by
    ``incidence`` degrees about y through ``origin`` and placed there."""
    xs = spacing(nc, "uniform")
    m, p = camber
    zc = naca4_camber(xs, m, p)
    pts = []
    for le, chord, twist in sections:
        loc = np.stack([xs * chord, np.zeros_like(xs), zc * chord], axis=1)
        pts.append(np.asarray(le, dtype=np.float64) + loc @ _rot_y(twist).T)
    st = spacing(ns, span_spacing)
    verts = (pts[0][:, None, :] * (1.0 - st)[None, :, None]
             + pts[1][:, None, :] * st[None, :, None])
    return np.asarray(origin, dtype=np.float64) + verts @ _rot_y(incidence).T


def mirror(verts, y0=0.0, join=True):
    """Mirror image of a right half wing about the plane y = y0, columns kept
    left -> right.  ``join``: the root column is shared (one continuous
    surface, 2 ns panels); else the mirror image alone is returned."""
    left = verts[:, ::-1, :].copy()
    left[:, :, 1] = 2 * y0 - left[:, :, 1]
    if join:
        return np.concatenate([left[:, :-1, :], verts], axis=1)
    return left


def combine(grids):
    """One vertex grid for several surfaces with the same nc: the grids side by
    side, with the strip -> vertex-column map ``col`` and the vertex-column ->
    surface map ``surf``."""
    nc = grids[0].shape[0] - 1
    assert all(g.shape[0] == nc + 1 for g in grids), "surfaces need the same nc"
    col, surf, c0 = [], [], 0
    for k, g in enumerate(grids):
        w = g.shape[1]
        col.extend(range(c0, c0 + w - 1))
        surf.extend([k] * w)
        c0 += w
    return (np.concatenate(grids, axis=1), np.asarray(col, dtype=np.int32),
            np.asarray(surf, dtype=np.int32))


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


def lattice(verts, col=None) -> Lattice:
    """Rings of strips j = 0..ns-1 between vertex columns col[j], col[j]+1
    (default: every adjacent column pair), ring k = i ns + j."""
    nc = verts.shape[0] - 1
    a = np.arange(verts.shape[1] - 1) if col is None else np.asarray(col)
    b = a + 1
    ns = a.size
    vq = np.empty_like(verts)
    vq[:-1] = verts[:-1] + 0.25 * (verts[1:] - verts[:-1])
    vq[-1] = verts[-1] + 0.25 * (verts[-1] - verts[-2])
    fl = vq[:-1, a].reshape(-1, 3)
    fr = vq[:-1, b].reshape(-1, 3)
    br = vq[1:, b].reshape(-1, 3)
    bl = vq[1:, a].reshape(-1, 3)
    vc = verts[:-1] + 0.75 * (verts[1:] - verts[:-1])
    colloc = (0.5 * (vc[:, a] + vc[:, b])).reshape(-1, 3)
    d1 = (verts[1:, b] - verts[:-1, a]).reshape(-1, 3)
    d2 = (verts[:-1, b] - verts[1:, a]).reshape(-1, 3)
    cr = np.cross(d1, d2)
    nrm = np.linalg.norm(cr, axis=1)
    return Lattice(br=np.ascontiguousarray(br), fr=np.ascontiguousarray(fr),
                   fl=np.ascontiguousarray(fl), bl=np.ascontiguousarray(bl),
                   colloc=np.ascontiguousarray(colloc), normal=cr / nrm[:, None],
                   area=0.5 * nrm, leg_center=0.5 * (fr + fl), leg_vec=fl - fr,
                   te_back=vq[-1].copy(), nc=nc, ns=ns)


@dataclass
class Kinematics:
    """Rigid motion of a surface: heave z(t) = h0 sin(2 pi t / T) and a
    flapping rotation theta(t) = A sin(2 pi t / T) about the x axis through the
    hinge lines y = +-y0, z = 0, each half wing (sign of y) about its own
    hinge, mirrored, so that both halves rotate up together."""
    heave_amp: float = 0.0
    flap_amp: float = 0.0          # radians
    period: float = 1.0
    y0: float = 0.0

    def vertices(self, base, t):
        v = base.copy()
        w = 2.0 * np.pi / self.period
        if self.flap_amp:
            th = self.flap_amp * np.sin(w * t)
            s = np.sign(v[..., 1])
            y, z = np.abs(v[..., 1]) - self.y0, v[..., 2]
            v[..., 1] = s * (self.y0 + (y * np.cos(th) - z * np.sin(th)))
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
        z plus the flapping rotation about the hinge line of the point's half
        wing, mirrored for the left half (v = s thetadot (0, -Z, dY), s = sign(y),
        dY = y - s y0)."""
        h, hdot, thdot = self.rates(t)
        p = np.asarray(p, dtype=np.float64)
        v = np.zeros_like(p)
        s = np.where(p[:, 1] >= 0.0, 1.0, -1.0)
        dy = p[:, 1] - s * self.y0
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
    # several surfaces (``combine``): strip -> vertex column, vertex column ->
    # surface, and each surface's motion; None = one surface moving with kin
    col: np.ndarray = None
    surf: np.ndarray = None
    kins: list = None
    s_ref: float = None            # CL / CDi reference area (None: sum of panel areas)
    # particle population control after each step's convection
    # (newton_pc/adapters/flap.py:264-279, 466-563): "none", "drop" (keep the
    # newest pop_max) or "merge" (one moment-conserving merge pass judged at 9
    # collocation points against merge_eps |V_inf|, the newest merge_protect
    # particles or those within merge_protect_dist of the wing excluded)
    # free ring wake: the kept ring rows move with the local velocity (bound
    # rings, wake rings, particles, freestream; PteraSoftware's free wake, cf.
    # newton_pc/adapters/flap.py:379-401) instead of the freestream alone
    free_ring_wake: bool = False
    # loads: "kj" (Kutta-Joukowski on the bound legs + unsteady term, the
    # PteraSoftware form) or "bernoulli" (unsteady Bernoulli pressure,
    # newton_pc/adapters/flap.py:357-377)
    loads: str = "kj"
    population: str = "none"
    pop_max: int = 60000
    merge_eps: float = 1e-3
    merge_protect: int = 64
    merge_protect_dist: float = None

    def ref_points(self, colloc):
        """The 9 wing reference points of the merge test: every (P // 9)-th
        collocation point (flap.py:426)."""
        P = colloc.shape[0]
        return colloc[:: max(1, P // 9)][:9]

    @property
    def speed(self):
        return float(np.linalg.norm(self.u_inf))

    def layout(self):
        """(col, surf, kins) with the one-surface defaults filled in."""
        w = self.verts.shape[1]
        col = np.arange(w - 1, dtype=np.int32) if self.col is None else self.col
        surf = np.zeros(w, dtype=np.int32) if self.surf is None else self.surf
        kins = [self.kin] if self.kins is None else self.kins
        return col, surf, kins

    def vertices(self, t):
        """The vertex grid at time t, each column moved by its surface."""
        col, surf, kins = self.layout()
        out = np.empty_like(self.verts)
        for k, kin in enumerate(kins):
            m = surf == k
            out[:, m] = kin.vertices(self.verts[:, m], t)
        return out

    def point_velocity(self, p, t):
        """Body velocity at panel points p (P,3), ring k = i ns + j moving with
        the surface of strip j."""
        col, surf, kins = self.layout()
        ps = surf[col]
        k_of = np.tile(ps, p.shape[0] // ps.size)
        v = np.zeros_like(p)
        for k, kin in enumerate(kins):
            m = k_of == k
            if m.any():
                v[m] = kin.point_velocity(p[m], t)
        return v


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


def flapping_aircraft(V=10.0, alpha_deg=1.0, period=1.0, flap_deg=15.0, steps_per_cycle=43,
                      n_keep=10, flapping="right", **kw) -> HybridConfig:
    """The large flapping configuration (tests/benchmark_flapping.py:28-141 of
    the FLUXVortex project, PteraSoftware's variable-geometry example):

    - main wing, NACA 2412: root chord 1.75 at the leading point (0, 0.5, 0),
      tip chord 1.5 with its leading point 0.75 aft, 6.0 out and 1.0 up,
      twisted 5 deg (trailing edge down); nc = 6, ns = 8 cosine; mirrored about
      y = 0 with its root 0.5 off the plane, so the two halves are separate
      surfaces; flapping 15 deg sin(2 pi t / 1 s) about the x axis through the
      root of the half;
    - V-tail, NACA 0012: root chord 1.5 at (5, 0, 0), tip chord 1.0 with its
      leading point 0.5 aft, 2.0 out and 1.0 up, the whole tail pitched -5 deg;
      nc = 6, ns = 8 uniform, mirrored about its root (one surface of 16
      strips), fixed;
    - V = 10 m/s at alpha = 1 deg; dt = period / 43 (the time step of the
      reference's saved histories, figures/flapping_results.npz).

    3 surfaces, 192 panels.  ``flapping="right"``: only the unreflected main
    half moves.  The benchmark selects the flapping wings by the name "Main
    Wing" (benchmark_flapping.py:117, :125-126) after PteraSoftware has split
    the main wing in two; the recorded CL history matches this form (one-step
    offset, correlation 0.999) and not the symmetric one, so the reflected
    half evidently does not keep the name.  ``"both"`` flaps the two halves
    symmetrically.  CL and CDi are on PteraSoftware's reference area for this
    airplane, the projected area of its first wing (the right main half), the
    normalisation of the recorded coefficients.  The panels follow
    PteraSoftware's lofting (linear between the two sections); PteraSoftware
    itself is absent, so the geometry is this restatement's, not bit-identical
    to its panels."""
    main = lofted_wing([((0.0, 0.0, 0.0), 1.75, 0.0), ((0.75, 6.0, 1.0), 1.5, 5.0)], 6, 8,
                       span_spacing="cosine", camber=(0.02, 0.4), origin=(0.0, 0.5, 0.0))
    tail = lofted_wing([((0.0, 0.0, 0.0), 1.5, 0.0), ((0.5, 2.0, 1.0), 1.0, 0.0)], 6, 8,
                       span_spacing="uniform", origin=(5.0, 0.0, 0.0), incidence=-5.0)
    verts, col, surf = combine([mirror(main, 0.0, join=False), main, mirror(tail, 0.0)])
    flap = Kinematics(flap_amp=np.radians(flap_deg), period=period, y0=0.5)
    fixed = Kinematics(period=period)
    if flapping not in ("right", "both"):
        raise ValueError(f"flapping must be 'right' or 'both', not {flapping!r}")
    kins = [flap if flapping == "both" else fixed, flap, fixed]
    # projected area of the right main half: its quadrilaterals' areas in xy
    q = main[:, :, :2]
    d1, d2 = q[1:, 1:] - q[:-1, :-1], q[:-1, 1:] - q[1:, :-1]
    s_ref = float(0.5 * np.abs(d1[..., 0] * d2[..., 1] - d1[..., 1] * d2[..., 0]).sum())
    a = np.radians(alpha_deg)
    return HybridConfig(verts=verts, u_inf=V * np.array([np.cos(a), 0.0, np.sin(a)]),
                        dt=period / steps_per_cycle, kin=flap, rc0=0.03 * 1.75, n_keep=n_keep,
                        col=col, surf=surf, kins=kins, s_ref=s_ref, **kw)
