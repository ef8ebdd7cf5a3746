"""Pins of the learned far-field oracle (CPU): network gradients against central
differences, exact local expansions against the quadrupole far field and a
Taylor step, BF16 rounding against torch's conversion."""
import numpy as np
import torch

from oracle import learned as OL
from oracle import treecode as TC


def _rand_net(seed, scale=0.3):
    rng = np.random.default_rng(seed)
    nw = sum(r * c for r, c in OL.LAYERS)
    nb = sum(r for r, _ in OL.LAYERS)
    return rng.standard_normal(nw) * scale, rng.standard_normal(nb) * 0.1


def test_bf16_rounding_matches_torch():
    rng = np.random.default_rng(1)
    x = np.concatenate([rng.standard_normal(4096) * 10.0 ** rng.integers(-6, 6, 4096),
                        [1.0 + 2.0 ** -8, 1.0 + 3 * 2.0 ** -8, -1.0 - 2.0 ** -8, 0.0]])
    ref = torch.tensor(x, dtype=torch.float32).to(torch.bfloat16).double().numpy()
    np.testing.assert_array_equal(OL.bf16(x), ref)


def test_gradients_match_central_differences():
    w, b = _rand_net(2)
    rng = np.random.default_rng(3)
    X = rng.standard_normal((5, OL.IN))
    T = rng.standard_normal((5, OL.OUT))
    loss, gw, gb = OL.gradients(w, b, X, T, rounding=False)
    scale = 1.0 / (X.shape[0] * OL.NOUT)
    eps = 1e-6
    for idx in list(rng.integers(0, w.size, 24)) + [OL.W_OFFSETS[3] + 5, OL.W_OFFSETS[0] + 3]:
        wp, wm = w.copy(), w.copy()
        wp[idx] += eps
        wm[idx] -= eps
        fd = (OL.gradients(wp, b, X, T, False)[0] - OL.gradients(wm, b, X, T, False)[0]) / (2 * eps)
        assert abs(fd * scale - gw[idx]) <= 1e-6 * max(1.0, abs(gw[idx])) + 1e-9, idx
    for idx in list(rng.integers(0, b.size, 12)) + [b.size - 1]:
        bp, bm = b.copy(), b.copy()
        bp[idx] += eps
        bm[idx] -= eps
        fd = (OL.gradients(w, bp, X, T, False)[0] - OL.gradients(w, bm, X, T, False)[0]) / (2 * eps)
        assert abs(fd * scale - gb[idx]) <= 1e-6 * max(1.0, abs(gb[idx])) + 1e-9, idx
    # padded output columns carry no gradient
    assert np.all(gb[OL.B_OFFSETS[3] + OL.NOUT:] == 0.0)


def test_local_expansion_matches_quadrupole_far_field():
    rng = np.random.default_rng(4)
    c = np.array([0.3, -0.2, 0.1])
    pos = c + rng.uniform(-0.05, 0.05, (40, 3))
    alpha = rng.standard_normal((40, 3))
    x0 = c + np.array([1.5, 0.7, -0.9])
    u, J, H = OL.local_expansion(x0, pos, alpha)
    d = pos - c
    M0 = alpha.sum(0)
    M1 = np.einsum("pm,pj->mj", alpha, d)
    M2 = np.einsum("pm,pj,pk->mjk", alpha, d, d)
    uq, Jq = TC.far_field(x0 - c, M0, M1, M2)
    # the quadrupole truncation error is O((r_S / d)^3) ~ 1e-4 here
    assert np.abs(u - uq).max() <= 2e-4 * np.abs(u).max()
    assert np.abs(J - Jq).max() <= 2e-4 * np.abs(J).max()
    assert np.allclose(H, np.swapaxes(H, 1, 2), rtol=0, atol=1e-14 * np.abs(H).max())


def test_local_expansion_taylor_step():
    rng = np.random.default_rng(5)
    pos = rng.uniform(-0.1, 0.1, (30, 3))
    alpha = rng.standard_normal((30, 3))
    x0 = np.array([1.2, 0.4, -0.5])
    u, J, H = OL.local_expansion(x0, pos, alpha)
    for k in range(3):
        e = np.zeros(3)
        e[k] = 1e-5
        up, Jp, _ = OL.local_expansion(x0 + e, pos, alpha)
        um, Jm, _ = OL.local_expansion(x0 - e, pos, alpha)
        np.testing.assert_allclose((up - um) / 2e-5, J[:, k], rtol=1e-6, atol=1e-8)
        np.testing.assert_allclose((Jp - Jm) / 2e-5, H[:, :, k], rtol=1e-6, atol=1e-8)
    # the divergence of a curl vanishes
    assert abs(np.trace(J)) <= 1e-12 * np.abs(J).max()


def test_pair_samples_consistent_with_tree():
    rng = np.random.default_rng(6)
    n = 3000
    pos = rng.uniform([0, 0, 0], [4.0, 2.0, 0.4], (n, 3))
    alpha = rng.standard_normal((n, 3)) * 1e-3
    tree = TC.build(pos, theta=0.5, leaf_target=16)
    pairs = OL.learned_pairs(tree, 0.5)
    far_total = sum(len(f) for _, f in TC.lists(tree))
    assert 0 < len(pairs) == far_total     # theta_learned = theta: every accepted cell
    fewer = OL.learned_pairs(tree, 0.35)
    assert 0 < len(fewer) < len(pairs)
    X, T = OL.pair_samples(tree, pos, alpha, pairs[::max(1, len(pairs) // 50)])
    np.testing.assert_allclose(np.linalg.norm(X[:, 0:3], axis=1), 1.0, rtol=1e-12)
    m = (np.linalg.norm(X[:, 5:8], axis=1) + np.linalg.norm(X[:, 8:17], axis=1)
         + np.sqrt((X[:, 17:35] ** 2 * np.tile([1, 2, 2, 1, 2, 1], 3)).sum(1)))
    np.testing.assert_allclose(m, 1.0, rtol=1e-12)
    assert np.all(X[:, OL.NFEAT:] == 0.0) and np.all(T[:, OL.NOUT:] == 0.0)
    assert np.all(np.isfinite(T)) and np.abs(T).max() < 1e3


def test_dtensor_closed_form_matches_explicit_tensors():
    r = np.array([0.7, -1.1, 0.4])
    D1, D2, D3, D4 = TC.phi_derivs(r)
    for p, D in ((1, D1), (2, D2), (3, D3), (4, D4)):
        np.testing.assert_allclose(OL.dtensor(r, p), D, rtol=1e-12, atol=1e-14)
    # the fifth derivative by central differences of the fourth
    D5 = OL.dtensor(r, 5)
    for k in range(3):
        e = np.zeros(3)
        e[k] = 1e-5
        fd = (OL.dtensor(r + e, 4) - OL.dtensor(r - e, 4)) / 2e-5
        np.testing.assert_allclose(D5[..., k], fd, rtol=1e-6, atol=1e-6 * np.abs(D5).max())


def test_m2l_converges_to_exact_local_expansion():
    rng = np.random.default_rng(7)
    c = np.array([0.2, 0.1, -0.3])
    pos = c + rng.uniform(-0.05, 0.05, (25, 3))
    alpha = rng.standard_normal((25, 3))
    errs = []
    for dist in (1.0, 2.0, 4.0):
        x0 = c + dist * np.array([0.6, -0.48, 0.64])
        exact = OL.pack_expansion(*OL.local_expansion(x0, pos, alpha))
        a = alpha * OL.KC
        d = pos - c
        M1 = np.einsum("pm,pj->mj", a, d)
        M2 = np.einsum("pm,pj,pk->mjk", a, d, d)
        approx = OL.pack_expansion(*OL.m2l(x0 - c, a.sum(0), M1, M2))
        errs.append(np.abs(approx - exact).max() / np.abs(exact).max())
    # octupole truncation: error ~ (r_S / d)^3, so x8 less per doubling
    assert errs[0] < 3e-3 and errs[1] < errs[0] / 5 and errs[2] < errs[1] / 5, errs


def test_m2l_from_features_matches_moments():
    rng = np.random.default_rng(8)
    pos = rng.uniform(-0.5, 0.5, (30, 3)) + np.array([0.0, 0.0, 0.0])
    alpha = rng.standard_normal((30, 3))
    cS, hS, cT, hT = np.zeros(3), 1.0, np.array([3.0, -2.0, 1.5]), 0.5
    M0, M1, M2 = OL.cell_moments(cS, pos, alpha)
    f, (s2, s3, s4) = OL.features(cT, hT, cS, hS, M0, M1, M2)
    got = OL.m2l_from_features(f)
    M1m = M1.reshape(3, 3)
    M2m = np.zeros((3, 3, 3))
    for m in range(3):
        for q, (j, k) in enumerate(OL.UNIQUE):
            M2m[m, j, k] = M2m[m, k, j] = M2[6 * m + q]
    ref = OL.pack_expansion(*OL.m2l(cT - cS, M0, M1m, M2m))
    np.testing.assert_allclose(got[0:3] * s2, ref[0:3], rtol=1e-10, atol=1e-14)
    np.testing.assert_allclose(got[3:12] * s3, ref[3:12], rtol=1e-10, atol=1e-14)
    np.testing.assert_allclose(got[12:30] * s4, ref[12:30], rtol=1e-10, atol=1e-14)


def test_dual_lists_partition_every_source_once():
    """The two-level lists reach every source particle from every target leaf
    exactly once (parent expansion, own expansion or near list)."""
    rng = np.random.default_rng(9)
    n = 4000
    pos = rng.uniform([0, 0, 0], [6.0, 3.0, 0.5], (n, 3))
    tree = TC.build(pos, theta=0.5, leaf_target=16)
    L = tree["L"]
    near, leaf_far, parent_far = TC.dual_lists(tree)
    levels = tree["levels"]
    leaves, parents = levels[L], levels[L - 1]
    assert sum(len(x) for x in parent_far) > 0 and sum(len(x) for x in leaf_far) > 0
    for t in range(len(leaves["start"])):
        p = int(np.searchsorted(parents["key"], leaves["key"][t] >> 3))
        cover = np.zeros(n, dtype=np.int64)
        for c in near[t]:
            cover[leaves["start"][c]:leaves["end"][c]] += 1
        for (l, c) in leaf_far[t] + parent_far[p]:
            cover[levels[l]["start"][c]:levels[l]["end"][c]] += 1
        assert np.all(cover == 1), t


def test_two_phase_lists_equal_per_leaf_lists():
    """The device's construction of the two-level lists (the walk once per
    parent, then each parent's residual cells against its leaves) gives the
    same sets as the per-leaf traversal, on a slab and on a clustered cloud."""
    rng = np.random.default_rng(13)
    clouds = [rng.uniform([0, 0, 0], [6.0, 3.0, 0.5], (3000, 3)),
              np.concatenate([rng.normal(0.0, 0.3, (1500, 3)),
                              rng.normal(2.0, 0.1, (1500, 3))])]
    for pos in clouds:
        tree = TC.build(pos, theta=0.5, leaf_target=16)
        a = TC.dual_lists(tree)
        b = TC.dual_lists_two_phase(tree)
        for la, lb in zip(a, b):
            assert len(la) == len(lb)
            for x, y in zip(la, lb):
                assert sorted(x) == sorted(y)


def _gen_m2l():
    import importlib.util
    import os
    path = os.path.join(os.path.dirname(__file__), "..", "fluxvortex_gb300", "csrc", "gen_m2l.py")
    spec = importlib.util.spec_from_file_location("gen_m2l", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_generated_m2l_matches_closed_form():
    """The straight-line multipole-to-local translation that the device runs
    (generated by csrc/gen_m2l.py) is the oracle's closed form: its FP64 twin
    from the same assignment list agrees to rounding on random unit offsets and
    moments."""
    G = _gen_m2l()
    f = G.python_twin()
    rng = np.random.default_rng(17)
    for _ in range(100):
        n = rng.standard_normal(3)
        n /= np.linalg.norm(n)
        feat = np.zeros(OL.IN)
        feat[0:3] = n
        feat[3] = rng.uniform(0.05, 0.7)
        feat[5:35] = rng.standard_normal(30)
        o = OL.m2l_from_features(feat)[:OL.NOUT]
        g = np.array(f(n, feat[5:8], feat[8:17], feat[17:35], feat[3]))
        assert np.abs(g - o).max() <= 1e-13 * np.abs(o).max()


def test_generated_m2l_header_is_current():
    """csrc/fvx_m2l_tensor.cuh is exactly what gen_m2l.py writes."""
    G = _gen_m2l()
    with open(G.OUT_H) as fh:
        assert fh.read() == G.cuda_source()
