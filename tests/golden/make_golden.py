"""Generate the golden vectors in this folder from the reference itself.

Run once, in a container that holds the FLUXVortex reference tree:

    python tests/golden/make_golden.py /root/reference

The reference's particle code (``src/fluxvortex/kernel.py``,
``src/fluxvortex/particles.py``) and beam model (``src/fluxvortex/beam_fe.py``)
import with NumPy/SciPy only and are called directly; its recorded flapping
histories (``figures/flapping_results.npz``) are copied as they are.  The reference's
line-vortex code (``src/fluxvortex/warp_kernels.py``) needs NVIDIA Warp, which
is not installed; this script registers a small pure-Python stand-in for the
``warp`` runtime (kernels run as Python functions, one call per thread id,
in thread-id order; ``wp.float64`` values are Python floats, i.e. IEEE
binary64 without FMA contraction; ``atomic_add`` is a plain add) and then
imports and calls the reference's own five public wrappers unchanged.  Nothing
of the reference is copied: its modules are executed in place.

The fixtures store inputs and outputs as ``.npz``; the tests read only these
files and never the reference tree.
"""
from __future__ import annotations

import math
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


# ---------------------------------------------------------------------------
# Pure-Python stand-in for the subset of the warp runtime that
# warp_kernels.py uses.

class _WArray:
    def __init__(self, data):
        self.data = data

    def __getitem__(self, i):
        v = self.data[i]
        if self.data.ndim == 2:
            return (float(v[0]), float(v[1]), float(v[2]))
        return float(v)

    def numpy(self):
        return self.data


def _install_warp_standin():
    wp = types.ModuleType("warp")
    state = {"tid": 0}

    class _Type:
        def __init__(self, name):
            self.name = name

        def __call__(self, *a):
            if self.name in ("float64", "float32"):
                return float(a[0])
            if self.name == "int32":
                return int(a[0])
            if self.name in ("vec3d", "vec3"):
                return tuple(float(x) for x in a)
            raise TypeError(self.name)

    for n in ("float64", "float32", "int32", "vec3d", "vec3"):
        setattr(wp, n, _Type(n))

    def array(data=None, dtype=None, **kw):
        if data is None:            # used as a type annotation
            return ("array", dtype)
        a = np.array(data, dtype=np.float64, copy=True)
        if getattr(dtype, "name", "") in ("vec3d", "vec3"):
            a = a.reshape(-1, 3)
        return _WArray(a)

    def zeros(n, dtype=None, **kw):
        if getattr(dtype, "name", "") in ("vec3d", "vec3"):
            return _WArray(np.zeros((n, 3)))
        return _WArray(np.zeros(n))

    def atomic_add(arr, idx, val):
        if arr.data.ndim == 2:
            arr.data[idx, 0] += val[0]
            arr.data[idx, 1] += val[1]
            arr.data[idx, 2] += val[2]
        else:
            arr.data[idx] += val

    def launch(kernel, dim, inputs, **kw):
        for t in range(int(dim)):
            state["tid"] = t
            kernel(*inputs)

    wp.array = array
    wp.zeros = zeros
    wp.atomic_add = atomic_add
    wp.launch = launch
    wp.tid = lambda: state["tid"]
    wp.sqrt = math.sqrt
    wp.abs = abs
    wp.kernel = lambda f: f
    wp.func = lambda f: f
    wp.init = lambda *a, **k: None
    sys.modules["warp"] = wp


# ---------------------------------------------------------------------------

def _ring_inputs(rng, N, M):
    """Inputs in the order of tests/test_correctness.py:19-31."""
    points = rng.standard_normal((N, 3))
    br = rng.standard_normal((M, 3))
    fr = rng.standard_normal((M, 3))
    fl = rng.standard_normal((M, 3))
    bl = rng.standard_normal((M, 3))
    strengths = rng.standard_normal(M) * 0.5
    rc0s = np.full(M, 0.03)
    ages = rng.uniform(0, 1, M)
    return points, br, fr, fl, bl, strengths, rc0s, ages, 1.5e-5


def _edge_inputs():
    """Degenerate geometry that exercises every skip test of
    warp_kernels.py:52,72-75,81: zero-length legs, points on ring corners,
    points on a leg's line, zero strengths."""
    rng = np.random.default_rng(7)
    M = 12
    br = rng.standard_normal((M, 3))
    fr = br + rng.standard_normal((M, 3))
    fl = fr + rng.standard_normal((M, 3))
    bl = fl + rng.standard_normal((M, 3))
    fr[0] = br[0]                       # zero-length BR->FR leg
    fl[1] = fr[1]                       # zero-length FR->FL leg
    bl[2] = br[2]                       # zero-length BL->BR leg
    strengths = rng.standard_normal(M)
    strengths[3] = 0.0
    rc0s = np.full(M, 0.03)
    rc0s[4] = 0.0                       # unregularised ring
    ages = rng.uniform(0, 2, M)
    pts = [br[5], fr[6], fl[7], bl[8],                  # on corners
           0.5 * (br[9] + fr[9]),                        # mid-leg
           br[10] + 2.5 * (fr[10] - br[10]),             # on the leg's line
           br[11] - 0.75 * (fr[11] - br[11]),            # on the line, behind
           fl[5] + 1e-13 * (fr[5] - fl[5]),              # within the tolerance
           ]
    pts = np.vstack([np.array(pts), rng.standard_normal((9, 3))])
    return pts, br, fr, fl, bl, strengths, rc0s, ages, 2.0e-5


def make_segments(ref_root):
    _install_warp_standin()
    sys.path.insert(0, os.path.join(ref_root, "src"))
    from fluxvortex import warp_kernels as wk  # noqa: E402  (reference module)

    fns = {
        "collapsed_ring": wk.collapsed_velocities_from_ring_vortices,
        "collapsed_ring_chordwise": wk.collapsed_velocities_from_ring_vortices_chordwise_segments,
        "expanded_ring": wk.expanded_velocities_from_ring_vortices,
        "collapsed_horseshoe": wk.collapsed_velocities_from_horseshoe_vortices,
        "expanded_horseshoe": wk.expanded_velocities_from_horseshoe_vortices,
    }
    cases = {
        # tests/test_correctness.py:19-31 (rng 42, N=200, M=100)
        "correctness": _ring_inputs(np.random.default_rng(42), 200, 100),
        "edge": _edge_inputs(),
    }
    for cname, (P, br, fr, fl, bl, s, rc, ages, nu) in cases.items():
        out = dict(points=P, br=br, fr=fr, fl=fl, bl=bl, strengths=s,
                   r_c0s=rc, ages=ages, nu=np.float64(nu))
        for fname, fn in fns.items():
            sing = np.zeros(4, dtype=np.int64)
            if "horseshoe" in fname:
                res = fn(P, br, fr, fl, bl, s, rc, sing, nu)
            else:
                res = fn(P, br, fr, fl, bl, s, rc, sing, ages, nu)
            out[fname] = np.array(res, dtype=np.float64)
            print(f"  segments/{cname}/{fname}: shape {out[fname].shape}")
        np.savez_compressed(os.path.join(HERE, f"segments_{cname}.npz"), **out)

    # warp_patch.benchmark() inputs (warp_patch.py:77-88), collapsed ring only,
    # at a reduced size so the pure-Python launch loop finishes in seconds.
    rng = np.random.default_rng(42)
    N, M = 120, 400
    P = rng.standard_normal((N, 3))
    br, fr, fl, bl = (rng.standard_normal((M, 3)) for _ in range(4))
    s = rng.standard_normal(M) * 0.5
    rc = np.full(M, 0.03)
    ages = rng.uniform(0, 1, M)
    res = wk.collapsed_velocities_from_ring_vortices(
        P, br, fr, fl, bl, s, rc, np.zeros(4, dtype=np.int64), ages, 1.5e-5)
    np.savez_compressed(os.path.join(HERE, "segments_benchmark_small.npz"),
                        points=P, br=br, fr=fr, fl=fl, bl=bl, strengths=s,
                        r_c0s=rc, ages=ages, nu=np.float64(1.5e-5),
                        collapsed_ring=np.array(res))
    print("  segments/benchmark_small done")

    # empty inputs (warp_kernels.py:193-194, 224-225)
    e3 = np.zeros((0, 3))
    r0 = wk.collapsed_velocities_from_ring_vortices(
        np.ones((5, 3)), e3, e3, e3, e3, np.zeros(0), np.zeros(0),
        np.zeros(4, dtype=np.int64))
    r1 = wk.expanded_velocities_from_ring_vortices(
        e3, np.ones((4, 3)), np.ones((4, 3)), np.ones((4, 3)), np.ones((4, 3)),
        np.ones(4), np.ones(4), np.zeros(4, dtype=np.int64))
    np.savez_compressed(os.path.join(HERE, "segments_empty.npz"),
                        collapsed_m0=r0, expanded_n0=r1)


def make_particles(ref_root):
    sys.path.insert(0, os.path.join(ref_root, "src"))
    from fluxvortex import kernel as K  # noqa: E402  (reference module)
    from fluxvortex.particles import VortexParticleField  # noqa: E402

    rng = np.random.default_rng(20261203)
    Ns, Mt = 700, 300
    pos = rng.uniform([0, -1, -0.2], [2, 1, 0.2], size=(Ns, 3))
    gam = rng.normal(0.0, 1e-3, size=(Ns, 3))
    sig = rng.uniform(0.02, 0.08, size=Ns)
    # targets: half of them coincide with sources (self pairs), half free
    tgt = np.vstack([pos[:Mt // 2], rng.uniform([0, -1, -0.2], [2, 1, 0.2], size=(Mt - Mt // 2, 3))])
    tgam = rng.normal(0.0, 1e-3, size=(Mt, 3))
    out = dict(src_pos=pos, src_gamma=gam, src_sigma=sig, tgt_pos=tgt, tgt_gamma=tgam)
    for kern in ("winckelmans", "gaussianerf"):
        out[f"velocity_{kern}"] = K.velocity_from_particles(tgt, pos, gam, sig, kernel=kern)
        out[f"jacobian_{kern}"] = K.jacobian_from_particles(tgt, tgam, pos, gam, sig, kernel=kern)
        print(f"  particles/{kern} done")
    np.savez_compressed(os.path.join(HERE, "particles_kernel.npz"), **out)

    # VortexParticleField.advect_rk3 (+ Pedrizzetti relaxation): two steps.
    n = 160
    p0 = rng.uniform([0, -1, -0.1], [1.5, 1, 0.1], size=(n, 3))
    g0 = rng.normal(0.0, 0.02, size=(n, 3))
    s0 = rng.uniform(0.05, 0.12, size=n)
    uinf = np.array([10.0, 0.0, -0.5])
    dt = 0.01
    res = dict(pos0=p0, gamma0=g0, sigma0=s0, u_inf=uinf, dt=np.float64(dt))
    for kern in ("winckelmans", "gaussianerf"):
        for stretch, free, rlxf in ((True, True, 0.3), (False, True, 0.3),
                                    (False, False, 0.3), (True, True, 0.0),
                                    (False, True, 0.0)):
            f = VortexParticleField(max_particles=n, nu=1e-4 if stretch else 0.0,
                                    rlxf=rlxf, kernel=kern)
            f.add_particles_batch(p0, g0, s0)
            for _ in range(2):
                f.advect_rk3(dt, lambda X: np.broadcast_to(uinf, X.shape).copy(),
                             stretch=stretch, free_wake=free)
            tag = f"{kern}_s{int(stretch)}_f{int(free)}_r{int(rlxf > 0)}"
            res[f"pos_{tag}"] = f.positions
            res[f"gamma_{tag}"] = f.gammas
            res[f"sigma_{tag}"] = f.sigmas
            res[f"age_{tag}"] = f._age[:f.np].copy()
            print(f"  particles/rk3 {tag} done")
    np.savez_compressed(os.path.join(HERE, "particles_rk3.npz"), **res)


def make_beam(ref_root):
    sys.path.insert(0, os.path.join(ref_root, "src"))
    from fluxvortex.beam_fe import BeamFE  # noqa: E402  (reference module)

    # Goland wing of the flutter sweep: 8 elements, EI/GJ/m/I_alpha per the
    # sweep's beam model, CG 0.183 m aft of the elastic axis.
    beam = BeamFE(length=6.096, n_elements=8, EI=9.773e6, GJ=0.988e6,
                  m_per_length=35.72, Ip=4.98, x_ea_cg=0.183)
    freqs, _ = beam.compute_natural_frequencies()
    F = np.zeros(beam.ndof)
    F[3::3] = 1000.0
    F[5::3] = 50.0
    hist = []
    for _ in range(5):
        beam.step(F, 0.003)
        hist.append(np.concatenate([beam.d, beam.v, beam.a]))
    np.savez_compressed(os.path.join(HERE, "beam_goland.npz"), freqs=freqs,
                        K=beam.K, M=beam.M, force=F, dt=np.float64(0.003),
                        history=np.array(hist))
    print("  beam done", freqs[:4])


def make_flapping(ref_root):
    """The reference's recorded CL / CDi histories of its flapping benchmark
    (figures/flapping_results.npz, written by tests/benchmark_flapping.py:251):
    PteraSoftware's ring wake and the hybrid N_keep = 10 run, 129 steps.  These
    are outputs of PteraSoftware geometry, so they pin the restated geometry
    qualitatively (correlation, mean, amplitude), not to round-off."""
    d = np.load(os.path.join(ref_root, "figures", "flapping_results.npz"), allow_pickle=False)
    np.savez_compressed(os.path.join(HERE, "flapping_history.npz"),
                        **{k: np.asarray(d[k], dtype=np.float64)
                           for k in ("t_ps", "cl_ps", "cdi_ps", "t_h10", "cl_h10", "cdi_h10")})
    print("  flapping done", d["cl_h10"].shape)


def _population_inputs(seed=11, n=3000):
    """A seeded wake-like cloud behind a unit wing: particles 0.2-12 chords
    downstream, strengths mostly along +y with noise (so that many cells hold
    aligned pairs), cores 0.05-0.25; 9 reference points on the wing."""
    rng = np.random.default_rng(seed)
    pos = np.column_stack([rng.uniform(0.2, 12.0, n), rng.uniform(-3.0, 3.0, n),
                           rng.normal(0.0, 0.3, n)])
    alpha = np.column_stack([rng.normal(0.0, 0.2, n), rng.normal(1.0, 0.5, n),
                             rng.normal(0.0, 0.2, n)]) * 1e-3
    sigma = rng.uniform(0.05, 0.25, n)
    ref = np.column_stack([np.full(9, 0.75), np.linspace(-2.5, 2.5, 9), np.zeros(9)])
    return pos, alpha, sigma, ref


def make_population(ref_root):
    """The reference's own merge pass (newton_pc/adapters/flap.py:478-563),
    called on a stand-in provider holding only the attributes it reads."""
    sys.path.insert(0, os.path.join(ref_root, "src"))
    sys.path.insert(0, ref_root)
    from newton_pc.adapters.flap import FlapUVLMProvider  # noqa: E402  (reference module)
    out = {}
    cases = {"count": dict(eps=1e-3, protect=64, dist=None),
             "dist": dict(eps=1e-3, protect=64, dist=3.0),
             "tight": dict(eps=1e-6, protect=200, dist=None)}
    for name, c in cases.items():
        pos, alpha, sigma, ref = _population_inputs()
        prov = types.SimpleNamespace(p_pos=pos.copy(), p_alpha=alpha.copy(), p_sigma=sigma.copy(),
                                     merge_protect=c["protect"], merge_eps=c["eps"],
                                     V_inf=np.array([10.0, 0.0, 0.0]),
                                     stats=dict(n_merged=0))
        if c["dist"]:
            prov.merge_protect_dist = c["dist"]
        FlapUVLMProvider._merge_pass(prov, ref)
        out.update({f"{name}_pos": prov.p_pos, f"{name}_alpha": prov.p_alpha,
                    f"{name}_sigma": prov.p_sigma,
                    f"{name}_merged": np.int64(prov.stats["n_merged"]),
                    f"{name}_eps": np.float64(c["eps"]), f"{name}_protect": np.int64(c["protect"]),
                    f"{name}_dist": np.float64(c["dist"] or 0.0)})
        print(f"  population {name}: {prov.stats['n_merged']} merges")
    pos, alpha, sigma, ref = _population_inputs()
    np.savez_compressed(os.path.join(HERE, "population_merge.npz"), pos=pos, alpha=alpha,
                        sigma=sigma, ref=ref, speed=np.float64(10.0), **out)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path of the FLUXVortex reference tree>")
    root = sys.argv[1]
    make_segments(root)
    make_particles(root)
    make_beam(root)
    make_flapping(root)
    make_population(root)
