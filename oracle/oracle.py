"""CPU oracle for the vortex-induction path (TEST INFRASTRUCTURE ONLY).

This module is the checker, never the product: only ``tests/``,
``__graft_entry__.smoke()`` and the ``cpu_baseline`` / ``--impl reference`` legs
of ``bench.py`` import it.  It wraps ``fvx_oracle.c`` (a plain-C FP64
restatement of the reference arithmetic, built with ``-ffp-contract=off`` and
OpenMP) and restates the reference's NumPy particle integrator.

Reference sources restated (paths inside the FLUXVortex project):
  * ``src/fluxvortex/warp_kernels.py:26-382`` -- the five PteraSoftware-signature
    Biot-Savart functions (line-vortex core law at :88);
  * ``src/fluxvortex/kernel.py:69-190`` -- particle velocity and Jacobian;
  * ``src/fluxvortex/particles.py:85-246`` -- RK3 + rVPM + relaxation;
  * ``tests/experiment_hybrid_panel_particle.py:145-204`` -- ring-row to
    particle conversion.

Parity pin: ``tests/golden/make_golden.py`` runs the reference's own Python
code (kernel.py and particles.py directly; warp_kernels.py's kernel bodies
through a pure-Python stand-in for the ``warp`` runtime) and stores the outputs
under ``tests/golden``; ``tests/test_oracle_golden.py`` checks this oracle
against them.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD = os.path.join(_HERE, "_build")
_SO = os.path.join(_BUILD, "libfvx_oracle.so")
_SRC = os.path.join(_HERE, "fvx_oracle.c")
_lock = threading.Lock()
_lib = None

LEGS_RING, LEGS_CHORDWISE, LEGS_HORSESHOE = 0, 1, 2
KERNELS = {"gaussianerf": 0, "winckelmans": 1}


def build(force: bool = False) -> str:
    """Compile ``fvx_oracle.c`` into ``oracle/_build/libfvx_oracle.so``."""
    os.makedirs(_BUILD, exist_ok=True)
    if (not force and os.path.exists(_SO)
            and os.path.getmtime(_SO) >= os.path.getmtime(_SRC)):
        return _SO
    tmp = _SO + f".tmp{os.getpid()}"
    cmd = ["gcc", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
           "-o", tmp, _SRC, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, _SO)
    return _SO


def _load():
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        lib = ctypes.CDLL(build())
        P = ctypes.c_void_p
        I64 = ctypes.c_int64
        D = ctypes.c_double
        I = ctypes.c_int
        for name in ("orc_segments_collapsed", "orc_segments_expanded"):
            f = getattr(lib, name)
            f.argtypes = [I64, P, I64, P, P, P, P, P, P, P, D, I, P, P]
            f.restype = I
        for name in ("orc_particle_velocity", "orc_particle_jacobian"):
            f = getattr(lib, name)
            f.argtypes = [I64, P, I64, P, P, P, I, P]
            f.restype = I
        lib.orc_particle_velocity_stretch.argtypes = [I64, P, P, I64, P, P, P, I, P, P]
        lib.orc_particle_velocity_stretch.restype = I
        lib.orc_num_threads.restype = I
        lib.orc_set_num_threads.argtypes = [I]
        _lib = lib
        return lib


def _c(a, dtype=np.float64):
    return np.ascontiguousarray(a, dtype=dtype)


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def num_threads() -> int:
    return _load().orc_num_threads()


def set_num_threads(n: int) -> None:
    _load().orc_set_num_threads(int(n))


# ---------------------------------------------------------------------------
# Line / ring / horseshoe Biot-Savart (warp_kernels.py:188-382)

def _segments(expanded, points, br, fr, fl, bl, strengths, r_c0s, counts, ages,
              nu, leg_set):
    points, br, fr, fl, bl = (_c(x).reshape(-1, 3) for x in (points, br, fr, fl, bl))
    strengths, r_c0s = _c(strengths).reshape(-1), _c(r_c0s).reshape(-1)
    N, M = points.shape[0], strengths.shape[0]
    ages = None if ages is None else _c(ages).reshape(-1)
    out = np.zeros((N, M, 3) if expanded else (N, 3))
    if N == 0 or M == 0:
        return out
    cnt = np.zeros(4, dtype=np.int64)
    fn = (_load().orc_segments_expanded if expanded
          else _load().orc_segments_collapsed)
    rc = fn(N, _p(points), M, _p(br), _p(fr), _p(fl), _p(bl), _p(strengths),
            _p(r_c0s), _p(ages), float(nu), leg_set, _p(out), _p(cnt))
    if rc != 0:
        raise ValueError("oracle: bad leg set")
    if counts is not None:
        counts += cnt
    return out


def collapsed_velocities_from_ring_vortices(P, Br, Fr, Fl, Bl, strengths, r_c0s,
                                            singularity_counts, ages=None, nu=0.0):
    return _segments(False, P, Br, Fr, Fl, Bl, strengths, r_c0s,
                     singularity_counts, ages, nu, LEGS_RING)


def collapsed_velocities_from_ring_vortices_chordwise_segments(
        P, Br, Fr, Fl, Bl, strengths, r_c0s, singularity_counts, ages=None, nu=0.0):
    return _segments(False, P, Br, Fr, Fl, Bl, strengths, r_c0s,
                     singularity_counts, ages, nu, LEGS_CHORDWISE)


def expanded_velocities_from_ring_vortices(P, Br, Fr, Fl, Bl, strengths, r_c0s,
                                           singularity_counts, ages=None, nu=0.0):
    return _segments(True, P, Br, Fr, Fl, Bl, strengths, r_c0s,
                     singularity_counts, ages, nu, LEGS_RING)


def collapsed_velocities_from_horseshoe_vortices(P, Br, Fr, Fl, Bl, strengths,
                                                 r_c0s, singularity_counts, nu=0.0):
    return _segments(False, P, Br, Fr, Fl, Bl, strengths, r_c0s,
                     singularity_counts, None, nu, LEGS_HORSESHOE)


def expanded_velocities_from_horseshoe_vortices(P, Br, Fr, Fl, Bl, strengths,
                                                r_c0s, singularity_counts, nu=0.0):
    return _segments(True, P, Br, Fr, Fl, Bl, strengths, r_c0s,
                     singularity_counts, None, nu, LEGS_HORSESHOE)


PS_FUNCTIONS = {
    "collapsed_velocities_from_ring_vortices": collapsed_velocities_from_ring_vortices,
    "collapsed_velocities_from_ring_vortices_chordwise_segments":
        collapsed_velocities_from_ring_vortices_chordwise_segments,
    "expanded_velocities_from_ring_vortices": expanded_velocities_from_ring_vortices,
    "collapsed_velocities_from_horseshoe_vortices":
        collapsed_velocities_from_horseshoe_vortices,
    "expanded_velocities_from_horseshoe_vortices":
        expanded_velocities_from_horseshoe_vortices,
}


# ---------------------------------------------------------------------------
# Vortex particles (kernel.py:69-190)

def velocity_from_particles(target_points, src_pos, src_gamma, src_sigma,
                            kernel="gaussianerf"):
    t = _c(target_points).reshape(-1, 3)
    s, g, sg = _c(src_pos).reshape(-1, 3), _c(src_gamma).reshape(-1, 3), _c(src_sigma).reshape(-1)
    out = np.zeros((t.shape[0], 3))
    if s.shape[0] == 0 or t.shape[0] == 0:
        return out
    _load().orc_particle_velocity(t.shape[0], _p(t), s.shape[0], _p(s), _p(g),
                                  _p(sg), KERNELS[kernel], _p(out))
    return out


def jacobian_from_particles(tgt_pos, tgt_gamma, src_pos, src_gamma, src_sigma,
                            kernel="gaussianerf"):
    t = _c(tgt_pos).reshape(-1, 3)
    s, g, sg = _c(src_pos).reshape(-1, 3), _c(src_gamma).reshape(-1, 3), _c(src_sigma).reshape(-1)
    out = np.zeros((t.shape[0], 3, 3))
    if s.shape[0] == 0 or t.shape[0] == 0:
        return out
    _load().orc_particle_jacobian(t.shape[0], _p(t), s.shape[0], _p(s), _p(g),
                                  _p(sg), KERNELS[kernel], _p(out))
    return out


def jacobian_reference_faithful(tgt_pos, src_pos, src_gamma, src_sigma,
                                kernel="gaussianerf"):
    """NumPy restatement of kernel.py:119-190 with SciPy's erf, as the reference
    evaluates it, including its cancellation of the Gaussian-erf core at
    r_bar -> 0 (kernel.py:16-31).  Used only to pin the reference's own
    numbers; everything else uses the series-corrected core of fvx_oracle.c."""
    from scipy.special import erf
    t = np.asarray(tgt_pos, dtype=np.float64).reshape(-1, 3)
    s = np.asarray(src_pos, dtype=np.float64).reshape(-1, 3)
    a = np.asarray(src_gamma, dtype=np.float64).reshape(-1, 3)
    sg = np.asarray(src_sigma, dtype=np.float64).reshape(-1)
    J = np.zeros((t.shape[0], 3, 3))
    if s.shape[0] == 0:
        return J
    C = -1.0 / (4.0 * np.pi)
    d = t[:, None, :] - s[None, :, :]
    r = np.sqrt(np.maximum(np.sum(d ** 2, axis=-1), 1e-24))
    rb = r / sg[None, :]
    if kernel == "gaussianerf":
        c = np.sqrt(2.0 / np.pi)
        ex = np.exp(-0.5 * rb ** 2)
        g = erf(rb / np.sqrt(2.0)) - c * rb * ex
        dg = c * rb ** 2 * ex
    else:
        r2 = rb ** 2
        g = rb ** 3 * (r2 + 2.5) / (r2 + 1.0) ** 2.5
        dg = 7.5 * r2 / (r2 + 1.0) ** 3.5
    r3inv = 1.0 / (r ** 3)
    KxG = C * np.cross(d, a[None, :, :]) * r3inv[:, :, None]
    aux = dg / (sg[None, :] * r) - 3.0 * g / (r ** 2)
    aux2 = C * g * r3inv
    # (row i, column j) -> (sign, strength component) of the aux2 term; each
    # entry is summed over sources as one expression, grouped as the
    # reference groups it (kernel.py:176-188), so rounding matches.
    skew = {(0, 1): (1, 2), (0, 2): (-1, 1), (1, 0): (-1, 2),
            (1, 2): (1, 0), (2, 0): (1, 1), (2, 1): (-1, 0)}
    for i in range(3):
        for j in range(3):
            term = aux * KxG[:, :, i] * d[:, :, j]
            if (i, j) in skew:
                sgn, k = skew[(i, j)]
                term = (term + aux2 * a[None, :, k] if sgn > 0
                        else term - aux2 * a[None, :, k])
            J[:, i, j] = np.sum(term, axis=1)
    return J


def velocity_and_stretching(tgt_pos, tgt_gamma, src_pos, src_gamma, src_sigma,
                            kernel="winckelmans"):
    """u (M,3) and S = J . Gamma_t (M,3) in one pass (particles.py:148-151)."""
    t = _c(tgt_pos).reshape(-1, 3)
    tg = _c(tgt_gamma).reshape(-1, 3)
    s, g, sg = _c(src_pos).reshape(-1, 3), _c(src_gamma).reshape(-1, 3), _c(src_sigma).reshape(-1)
    u = np.zeros((t.shape[0], 3))
    S = np.zeros((t.shape[0], 3))
    if s.shape[0] == 0 or t.shape[0] == 0:
        return u, S
    _load().orc_particle_velocity_stretch(t.shape[0], _p(t), _p(tg), s.shape[0],
                                          _p(s), _p(g), _p(sg), KERNELS[kernel],
                                          _p(u), _p(S))
    return u, S


# ---------------------------------------------------------------------------
# Particle field integrator (particles.py:85-246)

RK3_COEFFS = ((0.0, 1.0 / 3.0), (-5.0 / 9.0, 15.0 / 16.0), (-153.0 / 128.0, 8.0 / 15.0))


def advect_rk3(pos, gamma, sigma, age, dt, u_inf, kernel="gaussianerf", nu=0.0,
               rlxf=0.3, stretch=True, free_wake=True, faithful=False):
    """One RK3 + rVPM step followed by Pedrizzetti relaxation.

    Restates ``VortexParticleField.advect_rk3`` (particles.py:85-199) and
    ``_relax_pedrizzetti`` (particles.py:202-246) for a uniform freestream
    ``u_inf`` (3,) and no bound-vortex velocity.  Returns new (pos, gamma,
    sigma, age) arrays; the inputs are not modified.
    """
    pos = np.array(pos, dtype=np.float64, copy=True)
    gamma = np.array(gamma, dtype=np.float64, copy=True)
    sigma = np.array(sigma, dtype=np.float64, copy=True)
    age = np.array(age, dtype=np.float64, copy=True)
    n = pos.shape[0]
    if n == 0:
        return pos, gamma, sigma, age
    rk_X = np.zeros((n, 3))
    rk_G = np.zeros((n, 3))
    rk_s = np.zeros(n)
    max_gamma_sq = 1e4
    for a, b in RK3_COEFFS:
        if free_wake:
            U = velocity_from_particles(pos, pos, gamma, sigma, kernel)
        else:
            U = np.zeros_like(pos)
        U = U + np.broadcast_to(np.asarray(u_inf, dtype=np.float64), pos.shape)
        speed = np.linalg.norm(U, axis=1)
        fast = speed > 50.0
        if np.any(fast):
            U[fast] *= (50.0 / speed[fast])[:, None]
        rk_X = a * rk_X + dt * U
        pos += b * rk_X
        if stretch:
            if faithful:
                J = jacobian_reference_faithful(pos, pos, gamma, sigma, kernel)
            else:
                J = jacobian_from_particles(pos, gamma, pos, gamma, sigma, kernel)
            S = np.einsum("tij,tj->ti", J, gamma)
            g2 = np.sum(gamma ** 2, axis=1)
            sdg = np.sum(S * gamma, axis=1)
            mask = g2 > 1e-20
            Z = np.zeros(n)
            Z[mask] = 0.2 * sdg[mask] / g2[mask]
            zmax = 10.0 / max(dt, 1e-10)
            Z = np.clip(Z, -zmax, zmax)
            dG = S - 3.0 * Z[:, None] * gamma
            ds = -sigma * Z
            if nu > 0:
                ds += nu / np.maximum(sigma, 1e-10)
            rk_G = a * rk_G + dt * dG
            rk_s = a * rk_s + dt * ds
            gamma += b * rk_G
            sigma += b * rk_s
            g2 = np.sum(gamma ** 2, axis=1)
            big = g2 > max_gamma_sq
            if np.any(big):
                gamma[big] *= np.sqrt(max_gamma_sq / g2[big])[:, None]
            sigma = np.clip(sigma, 1e-6, 5.0)
    bad = ~np.isfinite(pos).all(axis=1) | ~np.isfinite(gamma).all(axis=1)
    if np.any(bad):
        gamma[bad] = 0.0
    age += dt
    gamma = relax_pedrizzetti(pos, gamma, sigma, rlxf, faithful)
    return pos, gamma, sigma, age


def relax_pedrizzetti(pos, gamma, sigma, rlxf, faithful=False):
    """particles.py:202-246 (always the Gaussian-erf Jacobian, :219).

    ``faithful=True`` evaluates that Jacobian exactly as the reference does
    (its self-pair term is then SciPy-erf rounding noise, see
    ``jacobian_reference_faithful``); the default uses the series-corrected
    core that the CUDA kernels implement."""
    gamma = np.array(gamma, dtype=np.float64, copy=True)
    if rlxf <= 0 or pos.shape[0] == 0:
        return gamma
    gn = np.linalg.norm(gamma, axis=1)
    active = gn > 1e-15
    if not np.any(active):
        return gamma
    if faithful:
        J = jacobian_reference_faithful(pos, pos, gamma, sigma, "gaussianerf")
    else:
        J = jacobian_from_particles(pos, gamma, pos, gamma, sigma, "gaussianerf")
    om = np.zeros_like(gamma)
    om[:, 0] = J[:, 2, 1] - J[:, 1, 2]
    om[:, 1] = J[:, 0, 2] - J[:, 2, 0]
    om[:, 2] = J[:, 1, 0] - J[:, 0, 1]
    on = np.linalg.norm(om, axis=1)
    mask = active & (on > 1e-12)
    if not np.any(mask):
        return gamma
    Gn = gn[mask]
    oh = om[mask] / on[mask, None]
    gamma[mask] = (1.0 - rlxf) * gamma[mask] + rlxf * Gn[:, None] * oh
    b2 = 1.0 - 2.0 * (1.0 - rlxf) * rlxf * (
        1.0 - np.sum(gamma[mask] * oh, axis=1) / np.maximum(Gn, 1e-12))
    b2 = np.maximum(b2, 0.01)
    gamma[mask] /= np.sqrt(b2)[:, None]
    return gamma


# ---------------------------------------------------------------------------
# Ring-row to particle conversion (experiment_hybrid_panel_particle.py:145-204)

def rings_to_particles(fr, fl, bl, br, strengths, sigma):
    """Four particles per ring (front, left, back, right legs).

    Rings with |strength| < 1e-15 are skipped (:179); a leg whose strength
    vector has |alpha|^2 <= 1e-30 emits no particle (:195).  Returns
    (pos (K,3), alpha (K,3), sigma (K,)) in ring-major, leg-minor order.
    """
    fr, fl, bl, br = (np.asarray(x, dtype=np.float64).reshape(-1, 3) for x in (fr, fl, bl, br))
    strengths = np.asarray(strengths, dtype=np.float64).reshape(-1)
    pos, alp = [], []
    for k in range(strengths.shape[0]):
        s = strengths[k]
        if abs(s) < 1e-15:
            continue
        legs = ((0.5 * (fr[k] + fl[k]), s * (fl[k] - fr[k])),
                (0.5 * (fl[k] + bl[k]), s * (bl[k] - fl[k])),
                (0.5 * (bl[k] + br[k]), s * (br[k] - bl[k])),
                (0.5 * (br[k] + fr[k]), s * (fr[k] - br[k])))
        for p, g in legs:
            if np.dot(g, g) > 1e-30:
                pos.append(p)
                alp.append(g)
    if not pos:
        return np.zeros((0, 3)), np.zeros((0, 3)), np.zeros(0)
    return np.array(pos), np.array(alp), np.full(len(pos), float(sigma))
