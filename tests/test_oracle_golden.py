"""The CPU oracle against golden vectors produced by the reference's own code
(tests/golden/make_golden.py).  CPU only."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.conftest import rel_err

SEG_FUNCS = {
    "collapsed_ring": O.collapsed_velocities_from_ring_vortices,
    "collapsed_ring_chordwise": O.collapsed_velocities_from_ring_vortices_chordwise_segments,
    "expanded_ring": O.expanded_velocities_from_ring_vortices,
    "collapsed_horseshoe": O.collapsed_velocities_from_horseshoe_vortices,
    "expanded_horseshoe": O.expanded_velocities_from_horseshoe_vortices,
}


def _seg_args(z):
    return [z[k] for k in ("points", "br", "fr", "fl", "bl", "strengths", "r_c0s")]


@pytest.mark.parametrize("case", ["correctness", "edge", "benchmark_small"])
@pytest.mark.parametrize("fname", list(SEG_FUNCS))
def test_segments_bit_exact(golden, case, fname):
    """The C restatement reproduces warp_kernels.py bit for bit (same operation
    order, no FMA contraction, same summation order)."""
    z = golden(f"segments_{case}.npz")
    if fname not in z:
        pytest.skip("fixture holds the collapsed ring only")
    cnt = np.zeros(4, np.int64)
    if "horseshoe" in fname:
        r = SEG_FUNCS[fname](*_seg_args(z), cnt, float(z["nu"]))
    else:
        r = SEG_FUNCS[fname](*_seg_args(z), cnt, z["ages"], float(z["nu"]))
    assert r.shape == z[fname].shape
    assert np.array_equal(r, z[fname])


def test_segments_edge_counts(golden):
    """The edge fixture trips every skip test of warp_kernels.py:52,72-75,81."""
    z = golden("segments_edge.npz")
    cnt = np.zeros(4, np.int64)
    O.collapsed_velocities_from_ring_vortices(*_seg_args(z), cnt, z["ages"], float(z["nu"]))
    assert np.all(cnt > 0), cnt


def test_segments_empty(golden):
    z = golden("segments_empty.npz")
    e3 = np.zeros((0, 3))
    r0 = O.collapsed_velocities_from_ring_vortices(np.ones((5, 3)), e3, e3, e3, e3, np.zeros(0),
                                                   np.zeros(0), np.zeros(4, np.int64))
    assert np.array_equal(r0, z["collapsed_m0"])
    r1 = O.expanded_velocities_from_ring_vortices(e3, *(np.ones((4, 3)),) * 4, np.ones(4),
                                                  np.ones(4), np.zeros(4, np.int64))
    assert r1.shape == z["expanded_n0"].shape


@pytest.mark.parametrize("kernel", ["winckelmans", "gaussianerf"])
def test_particle_velocity(golden, kernel):
    z = golden("particles_kernel.npz")
    u = O.velocity_from_particles(z["tgt_pos"], z["src_pos"], z["src_gamma"], z["src_sigma"],
                                  kernel)
    assert rel_err(u, z[f"velocity_{kernel}"]) < 1e-13


@pytest.mark.parametrize("kernel", ["winckelmans", "gaussianerf"])
def test_particle_jacobian(golden, kernel):
    """Targets 150.. are not sources: every pair is well conditioned and the
    series-corrected oracle matches the reference.  Targets 0..149 coincide
    with sources; there the reference-faithful form matches exactly, and for
    the Gaussian-erf core the reference's self-pair value is rounding noise
    (kernel.py:16-18 cancels at r = 1e-12), which the corrected core
    replaces by the analytic limit."""
    z = golden("particles_kernel.npz")
    G = z[f"jacobian_{kernel}"]
    J = O.jacobian_from_particles(z["tgt_pos"], z["tgt_gamma"], z["src_pos"], z["src_gamma"],
                                  z["src_sigma"], kernel)
    assert rel_err(J[150:], G[150:]) < 1e-13
    Jf = O.jacobian_reference_faithful(z["tgt_pos"], z["src_pos"], z["src_gamma"],
                                       z["src_sigma"], kernel)
    assert rel_err(Jf, G) < 1e-13
    if kernel == "winckelmans":
        assert rel_err(J, G) < 1e-13
    else:
        assert np.abs(G[:150]).max() > 1e3 * np.abs(G[150:]).max()   # the noise


def test_gaussian_series_matches_direct_where_both_accurate():
    from scipy.special import erf
    rb = np.linspace(0.3, 0.7, 41)
    c = np.sqrt(2 / np.pi)
    direct = erf(rb / np.sqrt(2)) - c * rb * np.exp(-0.5 * rb ** 2)
    # series of fvx_oracle.c through the velocity of one particle at distance rb
    for r, d in zip(rb, direct):
        u = O.velocity_from_particles(np.array([[r, 0, 0]]), np.zeros((1, 3)),
                                      np.array([[0, 0, 1.0]]), np.array([1.0]), "gaussianerf")
        expect = -1 / (4 * np.pi) * d / r ** 3 * (-r)   # d x alpha, y-component
        assert abs(u[0, 1] - expect) <= 5e-14 * abs(expect)


RK3_CASES = [("winckelmans", 1, 1, 1), ("winckelmans", 0, 1, 1), ("winckelmans", 0, 0, 1),
             ("winckelmans", 1, 1, 0), ("winckelmans", 0, 1, 0), ("gaussianerf", 0, 1, 1),
             ("gaussianerf", 0, 0, 1), ("gaussianerf", 1, 1, 0), ("gaussianerf", 0, 1, 0)]


@pytest.mark.parametrize("kernel,s,f,r", RK3_CASES)
def test_rk3_reference_faithful(golden, kernel, s, f, r):
    """Two VortexParticleField.advect_rk3 steps (particles.py:85-246)."""
    z = golden("particles_rk3.npz")
    tag = f"{kernel}_s{s}_f{f}_r{r}"
    p, g, sg, a = z["pos0"], z["gamma0"], z["sigma0"], np.zeros(len(z["sigma0"]))
    for _ in range(2):
        p, g, sg, a = O.advect_rk3(p, g, sg, a, float(z["dt"]), z["u_inf"], kernel,
                                   1e-4 if s else 0.0, 0.3 if r else 0.0, bool(s), bool(f),
                                   faithful=True)
    assert rel_err(p, z["pos_" + tag]) < 1e-14
    assert rel_err(g, z["gamma_" + tag]) < 1e-12
    assert rel_err(sg, z["sigma_" + tag]) < 1e-12
    assert np.array_equal(a, z["age_" + tag])


@pytest.mark.parametrize("kernel", ["winckelmans", "gaussianerf"])
def test_rk3_corrected_equals_faithful_without_relaxation(golden, kernel):
    """With relaxation off and the Winckelmans core (or no stretching) the
    corrected core changes nothing the reference computes."""
    z = golden("particles_rk3.npz")
    s = 1 if kernel == "winckelmans" else 0
    tag = f"{kernel}_s{s}_f1_r0"
    p, g, sg, a = z["pos0"], z["gamma0"], z["sigma0"], np.zeros(len(z["sigma0"]))
    for _ in range(2):
        p, g, sg, a = O.advect_rk3(p, g, sg, a, float(z["dt"]), z["u_inf"], kernel,
                                   1e-4 if s else 0.0, 0.0, bool(s), True)
    assert rel_err(p, z["pos_" + tag]) < 1e-14
    assert rel_err(g, z["gamma_" + tag]) < 1e-12


def test_beam_frequencies(golden):
    """Known answer for the flutter sweep's beam: Goland wing 7.695/21.14 Hz."""
    z = golden("beam_goland.npz")
    f = z["freqs"]
    assert abs(f[0] - 7.695) < 5e-3 and abs(f[1] - 21.14) < 5e-3


def test_beam_oracle_matches_reference_model(golden):
    """The restated beam (matrices, Newmark history) against the reference's BeamFE."""
    from oracle.beam import Beam
    z = golden("beam_goland.npz")
    b = Beam(length=6.096, n_elements=8, EI=9.773e6, GJ=0.988e6, m_per_length=35.72, Ip=4.98,
             x_ea_cg=0.183)
    np.testing.assert_allclose(b.K, z["K"], rtol=1e-14, atol=1e-14 * np.abs(z["K"]).max())
    np.testing.assert_allclose(b.M, z["M"], rtol=1e-14, atol=1e-14 * np.abs(z["M"]).max())
    np.testing.assert_allclose(b.frequencies(), z["freqs"], rtol=1e-10)
    for k in range(z["history"].shape[0]):
        b.step(z["force"], float(z["dt"]))
        got = np.concatenate([b.d, b.v, b.a])
        ref = z["history"][k]
        assert np.abs(got - ref).max() <= 1e-9 * np.abs(ref).max()


@pytest.mark.parametrize("case", ["count", "dist", "tight"])
def test_population_merge_matches_reference(golden, case):
    """The oracle's merge pass against the reference's own (flap.py:478-563)
    on a seeded wake-like cloud: same merges, bitwise the same particles."""
    from oracle import population as POP
    z = golden("population_merge.npz")
    n = z["sigma"].shape[0]
    p, a, s, _, m = POP.merge_pass(z["pos"], z["alpha"], z["sigma"], np.arange(n, dtype=float),
                                   z["ref"], float(z["speed"]), float(z[case + "_eps"]),
                                   int(z[case + "_protect"]), float(z[case + "_dist"]) or None)
    assert m == int(z[case + "_merged"]) > 0
    assert np.array_equal(p, z[case + "_pos"])
    assert np.array_equal(a, z[case + "_alpha"])
    assert np.array_equal(s, z[case + "_sigma"])
    # moment conservation: the total strength is unchanged up to rounding
    assert np.abs(a.sum(0) - z["alpha"].sum(0)).max() < 1e-15 * n


def test_population_drop_keeps_the_newest():
    from oracle import population as POP
    n = 10
    pos = np.arange(3 * n, dtype=float).reshape(n, 3)
    out = POP.drop_oldest(pos, pos, np.arange(n, dtype=float), np.arange(n, dtype=float), 4)
    assert np.array_equal(out[2], [6.0, 7.0, 8.0, 9.0])
    same = POP.drop_oldest(pos, pos, np.arange(n, dtype=float), np.arange(n, dtype=float), 20)
    assert same[0].shape[0] == n


@pytest.mark.parametrize("kernel", ["winckelmans", "gaussianerf"])
def test_numpy_restatement_of_the_reference_kernels(golden, kernel):
    """The NumPy restatement timed as the reference's CPU path gives the
    reference's own outputs (blocks of 512 over 300 targets x 700 sources:
    two source blocks, one partial)."""
    from oracle import numpy_reference as NR
    z = golden("particles_kernel.npz")
    u = NR.velocity_from_particles(z["tgt_pos"], z["src_pos"], z["src_gamma"], z["src_sigma"],
                                   kernel)
    assert rel_err(u, z[f"velocity_{kernel}"]) < 1e-13
    J = NR.jacobian_from_particles(z["tgt_pos"], z["src_pos"], z["src_gamma"], z["src_sigma"],
                                   kernel)
    assert rel_err(J, z[f"jacobian_{kernel}"]) < 1e-12
