"""Learned far-field operator on the GPU: the tcgen05 training GEMM, the MLP
forward and backward against the CPU oracle (gradient check), the sampled
training pairs against exact FP64 local expansions, and training."""
import ctypes

import numpy as np
import pytest
import torch

from oracle import learned as OL
from oracle import treecode as TC

pytestmark = pytest.mark.gpu


def _lib():
    from fluxvortex_gb300 import _capi
    return _capi


@pytest.mark.parametrize("tA,tB,M,N,K,split", [(0, 0, 128, 128, 128, 1), (1, 1, 32, 128, 1000, 3),
                                              (0, 1, 300, 128, 32, 1), (1, 1, 128, 48, 4096, 4),
                                              (1, 0, 200, 80, 130, 2)])
def test_tc_gemm_matches_fp32(cuda, tA, tB, M, N, K, split):
    capi = _lib()
    lib = capi.load()
    g = torch.Generator().manual_seed(M * 7 + N + K)
    a = torch.randn((K, M) if tA else (M, K), generator=g).to(torch.bfloat16)
    b = torch.randn((K, N) if tB else (N, K), generator=g).to(torch.bfloat16)
    A, B = a.cuda(), b.cuda()
    C = torch.zeros((M, N), dtype=torch.float32, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    capi.check(lib.fvx_mlp_gemm(A.data_ptr(), A.shape[1], tA, B.data_ptr(), B.shape[1], tB,
                                C.data_ptr(), N, M, N, K, split, 1 if split > 1 else 0, st))
    opA = a.float().T if tA else a.float()
    opB = b.float() if tB else b.float().T
    ref = (opA.double() @ opB.double())
    err = (C.cpu().double() - ref).abs().max() / ref.abs().max()
    assert err < 1e-5, err
    assert capi.status_read_and_clear() == 0


def _net(seed):
    from fluxvortex_gb300 import learned as L
    w, b = L.init_weights(seed)
    rng = np.random.default_rng(seed)
    b = (rng.standard_normal(b.size) * 0.1).astype(np.float32)
    return L.FarFieldMLP(w, b)


def test_mlp_inference_form_matches_oracle(cuda):
    """The far field's inference form (no stores: packed BF16 SiLU on halved
    weights) against the oracle's restatement with the same BF16 rounding
    points, with the trained weights on pair features of a slab wake; and its
    distance from the unrounded FP64 network, the price of the BF16 form."""
    from fluxvortex_gb300 import learned as L
    from fluxvortex_gb300.tree import TreeSweeper
    from fluxvortex_gb300.workloads import slab_wake
    m = L.FarFieldMLP.load()
    pos, gam, sig, _ = slab_wake(1 << 15, seed=31)
    d = lambda a: torch.tensor(a, dtype=torch.float64, device="cuda")  # noqa: E731
    ts = TreeSweeper(theta=0.5, leaf_target=32)
    X, T, A = L.harvest(ts, d(pos), d(gam), d(sig), 1 << 15, 4000)
    rows = X.shape[0]
    assert rows >= 1000
    Y = m.forward(X).cpu().numpy()
    w, b = m.weights_numpy()
    Xh = X.float().cpu().numpy()
    Yo = OL.forward_inference(w, b, Xh)
    Y64, _ = OL.forward(w, b, Xh, rounding=False)
    scale = np.abs(Yo[:, :L.NOUT]).max()
    err = np.abs(Y[:, :L.NOUT] - Yo[:, :L.NOUT]).max() / scale
    e64 = np.abs(Y[:, :L.NOUT] - Y64[:, :L.NOUT]).max() / scale
    # the residual's share of the expansion it corrects
    share = float((torch.tensor(Y[:, :L.NOUT]).norm(dim=1)
                   / T[:, :L.NOUT].cpu().norm(dim=1).clamp_min(1e-30)).median())
    print(f"inference form vs oracle {err:.3e}, vs unrounded FP64 network {e64:.3e}; "
          f"median |residual| / |expansion| {share:.3e}")
    assert err < 2e-2, err
    assert e64 < 5e-2, e64
    assert _lib().status_read_and_clear() == 0


def test_mlp_forward_matches_oracle(cuda):
    from fluxvortex_gb300 import learned as L
    m = _net(11)
    rng = np.random.default_rng(12)
    rows = 1000                      # 8 tiles, the last one partial
    X = np.zeros((rows, L.IN), np.float32)
    X[:, :L.NFEAT] = rng.standard_normal((rows, L.NFEAT))
    Xd = torch.tensor(X).to(torch.bfloat16).cuda()
    Y, Z, Hs = m.forward(Xd, store=True)
    w, b = m.weights_numpy()
    Yo, (Zo, Ho) = OL.forward(w, b, Xd.float().cpu().numpy())
    Y = Y.cpu().numpy()
    err = np.abs(Y[:, :L.NOUT] - Yo[:, :L.NOUT]).max() / np.abs(Yo[:, :L.NOUT]).max()
    assert err < 1e-2, err
    zerr = np.abs(Z.cpu().numpy()[0] - Zo[0]).max() / np.abs(Zo[0]).max()
    assert zerr < 1e-5, zerr          # first layer: same BF16 operands, FP32 accumulation
    assert torch.isfinite(Hs.float()).all()
    assert _lib().status_read_and_clear() == 0


def test_mlp_gradients_match_oracle(cuda):
    """Gradient check: tensor-core backward against the FP64 oracle with the same
    BF16 rounding points."""
    from fluxvortex_gb300 import learned as L
    m = _net(21)
    rng = np.random.default_rng(22)
    rows = 2048
    X = np.zeros((rows, L.IN), np.float32)
    X[:, :L.NFEAT] = rng.standard_normal((rows, L.NFEAT))
    T = np.zeros((rows, L.OUT), np.float32)
    T[:, :L.NOUT] = rng.standard_normal((rows, L.NOUT))
    Xd = torch.tensor(X).to(torch.bfloat16).cuda()
    Td = torch.tensor(T).cuda()
    loss, _ = m.gradients(Xd, Td)
    w, b = m.weights_numpy()
    lo, gwo, gbo = OL.gradients(w, b, Xd.float().cpu().numpy(), T)
    assert abs(float(loss.item()) - lo) <= 1e-3 * lo
    gw, gb = m.gw.cpu().numpy(), m.gb.cpu().numpy()
    for li, ((r, c), o) in enumerate(zip(L.LAYERS, L.W_OFFSETS)):
        a, e = gw[o:o + r * c], gwo[o:o + r * c]
        rel = np.abs(a - e).max() / np.abs(e).max()
        assert rel < 2e-2, (li, rel)
        cos = float(a @ e / (np.linalg.norm(a) * np.linalg.norm(e)))
        assert cos > 0.9995, (li, cos)
    for li, ((r, _), o) in enumerate(zip(L.LAYERS, L.B_OFFSETS)):
        a, e = gb[o:o + r], gbo[o:o + r]
        rel = np.abs(a - e).max() / np.abs(e).max()
        assert rel < 2e-2, (li, rel)
    assert _lib().status_read_and_clear() == 0


def _slab(n, seed):
    rng = np.random.default_rng(seed)
    pos = rng.uniform([0, 0, 0], [4.0, 2.0, 0.4], (n, 3))
    alpha = rng.standard_normal((n, 3)) * 1e-3
    sigma = np.full(n, 0.02)
    return pos, alpha, sigma


def test_sampled_pairs_match_exact_local_expansions(cuda):
    from fluxvortex_gb300.tree import TreeSweeper
    from fluxvortex_gb300 import _capi
    n, leaf = 6000, 16
    pos, alpha, sigma = _slab(n, 31)
    ts = TreeSweeper(theta=0.5, leaf_target=leaf)
    ts.set_far_field("m2l", theta_local=0.4)
    d = lambda a: torch.tensor(a, dtype=torch.float64, device="cuda")  # noqa: E731
    out = torch.empty((n, 3), dtype=torch.float64, device="cuda")
    stats = ts.sweep(_capi.PAIR_VELOCITY, "winckelmans", d(pos), d(alpha), d(sigma), n, out,
                     check=True)
    tree = TC.build(pos, theta=0.5, leaf_target=leaf)
    pairs = OL.learned_pairs(tree, 0.4)
    assert int(stats[4]) == len(pairs) > 0
    max_pairs = 97
    Xg, Tg, Ag = ts.sample_pairs(max_pairs)
    stride = len(pairs) // max_pairs if len(pairs) > max_pairs else 1
    k = min(len(pairs) // stride, max_pairs)
    assert Xg.shape[0] == k
    Xo, To = OL.pair_samples(tree, pos, alpha, [pairs[i * stride] for i in range(k)])
    Xg = Xg.float().cpu().numpy()
    Tg = Tg.cpu().numpy()
    Ag = Ag.cpu().numpy()
    # features: the device's BF16 rounding of FP32 values, one BF16 step at most
    assert np.all(np.abs(Xg - Xo) <= 2.0 ** -7 * np.abs(Xo) + 1e-6)
    # targets: FP64 sums of FP32 particle offsets
    rel = np.abs(Tg - To).max(axis=1) / np.abs(To).max(axis=1)
    assert rel.max() < 1e-4, rel.max()
    # analytic multipole-to-local translation: FP32 device vs FP64 closed form
    Ao = np.stack([OL.m2l_from_features(x) for x in Xo])
    rel = np.abs(Ag - Ao).max(axis=1) / np.abs(Ao).max(axis=1)
    assert rel.max() < 1e-4, rel.max()
    # and it approximates the exact expansion to the quadrupole's truncation
    assert np.median(np.linalg.norm(Ao - To, axis=1) / np.linalg.norm(To, axis=1)) < 0.05
    assert _capi.status_read_and_clear() == 0


def test_training_reduces_loss(cuda):
    from fluxvortex_gb300 import learned as L
    from fluxvortex_gb300.tree import TreeSweeper
    n = 60000
    pos, alpha, sigma = _slab(n, 41)
    d = lambda a: torch.tensor(a, dtype=torch.float64, device="cuda")  # noqa: E731
    ts = TreeSweeper(theta=0.5, leaf_target=32)
    X, T, A = L.harvest(ts, d(pos), d(alpha), d(sigma), n, 40000)
    assert X.shape[0] > 10000
    # a network fitting the exact expansion itself learns fast from scratch
    m = L.FarFieldMLP(seed=3)
    Z = torch.zeros_like(A)
    e0 = float(m.errors(X, T, Z).median())
    hist = m.fit(X, T, steps=400, batch=4096, lr=2e-3, log_every=100)
    e1 = float(m.errors(X, T, Z).median())
    assert hist[-1][1] < 0.2 * hist[0][1], hist
    assert e1 < 0.5 * e0, (e0, e1)
    # the residual network starts at the analytic translation's accuracy
    r = L.FarFieldMLP(seed=4)
    ea = float(L.analytic_errors(T, A).median())
    er = float(r.errors(X, T, A).median())
    assert abs(er - ea) < 0.05 * ea, (er, ea)
    assert _lib().status_read_and_clear() == 0


def test_sampled_parent_pairs_match_exact_local_expansions(cuda):
    """Pairs shared through parents of leaves (two-level lists): features and
    FP64 targets about the parent's centre against the oracle."""
    from fluxvortex_gb300.tree import TreeSweeper
    from fluxvortex_gb300 import _capi
    n, leaf = 6000, 16
    pos, alpha, sigma = _slab(n, 33)
    ts = TreeSweeper(theta=0.5, leaf_target=leaf)
    ts.set_far_field("m2l")
    ts.set_validation(0, 0.1)
    d = lambda a: torch.tensor(a, dtype=torch.float64, device="cuda")  # noqa: E731
    out = torch.empty((n, 3), dtype=torch.float64, device="cuda")
    ts.sweep(_capi.PAIR_VELOCITY, "winckelmans", d(pos), d(alpha), d(sigma), n, out)
    tree = TC.build(pos, theta=0.5, leaf_target=leaf)
    _, _, parent_far = TC.dual_lists(tree)
    pairs = [(p, l, c) for p, lst in enumerate(parent_far) for (l, c) in lst]
    assert len(pairs) > 0
    max_pairs = 61
    Xg, Tg, Ag = ts.sample_pairs(max_pairs, parents=True)
    stride = len(pairs) // max_pairs if len(pairs) > max_pairs else 1
    k = min(len(pairs) // stride, max_pairs)
    assert Xg.shape[0] == k
    Xg, Tg = Xg.float().cpu().numpy(), Tg.cpu().numpy()
    # a parent's list is a set; its order on the device is the device's own.
    # Each sampled device pair is matched to the oracle pair whose features it
    # rounds (BF16), the matches must be distinct, and their FP64 targets agree
    Xall = OL.pair_features(tree, pos, alpha, pairs, target_level=tree["L"] - 1)
    idx = []
    for x in Xg:
        excess = (np.abs(Xall - x) - (2.0 ** -7 * np.abs(Xall) + 1e-6)).max(axis=1)
        j = int(np.argmin(excess))
        assert excess[j] <= 0.0, excess[j]
        idx.append(j)
    assert len(set(idx)) == len(idx)
    Xo, To = OL.pair_samples(tree, pos, alpha, [pairs[j] for j in idx],
                             target_level=tree["L"] - 1)
    assert np.all(np.abs(Xg - Xo) <= 2.0 ** -7 * np.abs(Xo) + 1e-6)
    rel = np.abs(Tg - To).max(axis=1) / np.abs(To).max(axis=1)
    assert rel.max() < 1e-4, rel.max()
    assert _capi.status_read_and_clear() == 0
