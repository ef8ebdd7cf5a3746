"""Treecode self-sweeps on the GPU.

1. Against the oracle's FP64 restatement of the same algorithm
   (oracle/treecode.py: same grid, sort, cells, lists, quadrupole far field):
   differences come from FP32 arithmetic only -> 2e-5 relative.
2. Against the direct FP64 sum: the approximation error of theta = 0.5 with
   quadrupole cells -> 1e-3 relative (velocity), 1e-2 (stretching,
   vorticity: one derivative more).
3. Degenerate inputs: one particle, fewer particles than a leaf, a planar sheet."""
import numpy as np
import pytest
import torch

from fluxvortex_gb300 import _capi
from fluxvortex_gb300 import kernel as K
from fluxvortex_gb300.tree import TreeSweeper
from fluxvortex_gb300.workloads import slab_wake
from oracle import treecode as OT
from tests.conftest import rel_err

pytestmark = pytest.mark.gpu


def _dev(a, cuda):
    return torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float64, device=cuda)


def _tree(mode, kernel, pos, gam, sig, cuda, leaf_target, theta=0.5, tg=None):
    n = pos.shape[0]
    ts = TreeSweeper(theta=theta, leaf_target=leaf_target)
    a = torch.empty((n, 3), dtype=torch.float64, device=cuda)
    b = torch.empty((n, 3), dtype=torch.float64, device=cuda) if mode == 2 else None
    stats = ts.sweep(mode, kernel, _dev(pos, cuda), _dev(gam, cuda), _dev(sig, cuda), n, a, b,
                     tgt_gamma=None if tg is None else _dev(tg, cuda), check=True)
    torch.cuda.synchronize()
    return a.cpu().numpy(), (None if b is None else b.cpu().numpy()), stats.copy()


@pytest.mark.parametrize("kernel", ["winckelmans", "gaussianerf"])
def test_tree_matches_oracle_algorithm(cuda, kernel):
    pos, gam, sig, _ = slab_wake(3000, seed=5)
    tr = OT.build(pos, theta=0.5, leaf_target=16)
    OT.moments(tr, pos, gam)
    u, J = OT.evaluate(tr, pos, gam, sig, kernel=kernel)
    S = np.einsum("tij,tj->ti", J, gam)
    w = np.stack([J[:, 2, 1] - J[:, 1, 2], J[:, 0, 2] - J[:, 2, 0], J[:, 1, 0] - J[:, 0, 1]], 1)
    gu, _, st = _tree(_capi.PAIR_VELOCITY, kernel, pos, gam, sig, cuda, 16)
    assert st[0] == tr["L"] and st[1] == len(tr["levels"][-1]["start"])
    lst = OT.lists(tr)
    assert st[2] == sum(len(a) for a, _ in lst) and st[3] == sum(len(b) for _, b in lst)
    assert rel_err(gu, u) < 2e-5
    gs, _, _ = _tree(_capi.PAIR_STRETCH, kernel, pos, gam, sig, cuda, 16, tg=gam)
    assert rel_err(gs, S) < 2e-5
    gw, _, _ = _tree(_capi.PAIR_VORTICITY, kernel, pos, gam, sig, cuda, 16)
    assert rel_err(gw, w) < 2e-5
    ga, gb, _ = _tree(_capi.PAIR_VELOCITY_STRETCH, kernel, pos, gam, sig, cuda, 16, tg=gam)
    assert rel_err(ga, u) < 2e-5 and rel_err(gb, S) < 2e-5


def test_tree_accuracy_vs_direct_fp64(cuda):
    pos, gam, sig, _ = slab_wake(1 << 16, seed=9)
    u64, _ = K.particle_pairs(_capi.PAIR_VELOCITY, _dev(pos, cuda), None, _dev(pos, cuda),
                              _dev(gam, cuda), _dev(sig, cuda), "winckelmans", "f64")
    s64, _ = K.particle_pairs(_capi.PAIR_STRETCH, _dev(pos, cuda), _dev(gam, cuda),
                              _dev(pos, cuda), _dev(gam, cuda), _dev(sig, cuda), "winckelmans",
                              "f64")
    gu, _, st = _tree(_capi.PAIR_VELOCITY, "winckelmans", pos, gam, sig, cuda, 64)
    gs, _, _ = _tree(_capi.PAIR_STRETCH, "winckelmans", pos, gam, sig, cuda, 64, tg=gam)
    assert st[3] > 0 and st[2] > 0
    assert rel_err(gu, u64.cpu().numpy()) < 1e-3
    assert rel_err(gs, s64.cpu().numpy()) < 1e-2


@pytest.mark.parametrize("case", ["one", "few", "sheet"])
def test_tree_degenerate_inputs(cuda, case):
    rng = np.random.default_rng(3)
    if case == "one":
        pos = np.array([[0.3, -0.2, 0.1]])
    elif case == "few":
        pos = rng.uniform(0, 1, (5, 3))
    else:
        pos = np.c_[rng.uniform(0, 4, (4000, 2)), np.full(4000, 0.25)]
    n = pos.shape[0]
    gam = rng.normal(0, 1e-3, (n, 3))
    sig = np.full(n, 0.05)
    gu, _, _ = _tree(_capi.PAIR_VELOCITY, "winckelmans", pos, gam, sig, cuda, 64)
    ud, _ = K.particle_pairs(_capi.PAIR_VELOCITY, pos, None, pos, gam, sig, "winckelmans", "f64")
    assert np.all(np.isfinite(gu))
    if np.abs(ud).max() > 0:
        # a planar sheet puts every far cell's quadrupole error in one plane
        assert rel_err(gu, ud) < (3e-3 if case == "sheet" else 1e-3)


@pytest.mark.parametrize("far", ["m2p", "learned"])
def test_reused_structure_matches_a_full_build(cuda, far):
    """A sweep hinted to have the last build's positions (new strengths and
    cores) equals a fresh full build: bitwise with the per-particle far field,
    within FP32 atomic-order noise with local expansions (their sums use
    atomics).  A hint with another particle count builds anew."""
    from fluxvortex_gb300.learned import FarFieldMLP
    pos, gam, sig, _ = slab_wake(1 << 15)
    rng = np.random.default_rng(3)
    gam2, sig2 = gam * rng.uniform(0.5, 1.5, gam.shape), sig * rng.uniform(0.8, 1.2, sig.shape)
    n = pos.shape[0]
    P, G, S = _dev(pos, cuda), _dev(gam, cuda), _dev(sig, cuda)
    G2, S2 = _dev(gam2, cuda), _dev(sig2, cuda)
    mlp = FarFieldMLP.load() if far == "learned" else None

    def sweeper():
        ts = TreeSweeper(theta=0.5, leaf_target=32)
        if far == "learned":
            ts.set_far_field("learned", mlp=mlp)
            ts.set_validation(0)
        return ts

    out = lambda: torch.empty((n, 3), dtype=torch.float64, device=cuda)  # noqa: E731
    ts = sweeper()
    first, reused = out(), out()
    ts.sweep(_capi.PAIR_STRETCH, "winckelmans", P, G, S, n, first, tgt_gamma=G)
    ts.sweep(_capi.PAIR_STRETCH, "winckelmans", P, G2, S2, n, reused, tgt_gamma=G2,
             same_positions=True)
    fresh = out()
    sweeper().sweep(_capi.PAIR_STRETCH, "winckelmans", P, G2, S2, n, fresh, tgt_gamma=G2)
    a, b = reused.cpu().numpy(), fresh.cpu().numpy()
    if far == "m2p":
        assert np.array_equal(a, b)
    else:
        assert np.abs(a - b).max() <= 1e-5 * np.abs(b).max()
    # the hint is ignored when the count changes
    m = n - 1000
    part, part_fresh = out(), out()
    ts.sweep(_capi.PAIR_STRETCH, "winckelmans", P, G2, S2, m, part, tgt_gamma=G2,
             same_positions=True)
    sweeper().sweep(_capi.PAIR_STRETCH, "winckelmans", P, G2, S2, m, part_fresh, tgt_gamma=G2)
    a, b = part[:m].cpu().numpy(), part_fresh[:m].cpu().numpy()
    tol = 0.0 if far == "m2p" else 1e-5 * np.abs(b).max()
    assert np.abs(a - b).max() <= tol
    assert _capi.status_read_and_clear() == 0


def test_one_pass_lists_and_their_overflow_fallback(cuda):
    """The two-level lists written in one pass into slots, with slots so small
    that they overflow (counting fallback), and with the counting pass only,
    give the same sweep."""
    pos, gam, sig, _ = slab_wake(1 << 15)
    n = pos.shape[0]
    P, G, S = _dev(pos, cuda), _dev(gam, cuda), _dev(sig, cuda)
    outs = []
    for slots in ((512, 1024, 1024), (4, 4, 4), (0, 0, 0)):
        ts = TreeSweeper(theta=0.5, leaf_target=32)
        ts.set_far_field("m2l")
        ts.set_validation(0)
        ts.set_list_slots(*slots)
        out = torch.empty((n, 3), dtype=torch.float64, device=cuda)
        stats = ts.sweep(_capi.PAIR_VELOCITY, "winckelmans", P, G, S, n, out, check=True).copy()
        outs.append((out.cpu().numpy(), stats))
    ref = outs[2][0]
    for o, st in outs[:2]:
        assert np.abs(o - ref).max() <= 1e-5 * np.abs(ref).max()
        assert np.array_equal(st[:5], outs[2][1][:5])


def _factored_case(n=3000, leaf=16, seed=5):
    """A slab whose cores are 1.3 x the particle spacing (the benchmarked
    step's), so that the leaves are at most four cores wide and the sweep
    takes the factored near loop (d x a = t x a - x_s x a)."""
    from fluxvortex_gb300.tree_params import grid_params
    from fluxvortex_gb300.workloads import resolved_core
    pos, gam, sig, _ = slab_wake(n, seed=seed, sigma=resolved_core(n))
    h = grid_params(pos.min(0), pos.max(0), n, leaf)["h"]
    assert h <= 4.0 * sig.min(), (h, sig.min())
    return pos, gam, sig


@pytest.mark.parametrize("n,leaf", [(3000, 16), (12000, 64)])
def test_factored_near_loop_matches_oracle_algorithm(cuda, n, leaf):
    """The factored velocity and stretching loops against the oracle's FP64
    restatement of the same treecode: the difference is the FP32 rounding
    (3.9e-7 measured for both; the bar is ten times that).  Leaf target 64
    gives leaves of more than 64 particles, which the velocity loop (four
    targets per lane, chunks of up to 64) takes in two chunks."""
    pos, gam, sig = _factored_case(n=n, leaf=leaf)
    tr = OT.build(pos, theta=0.5, leaf_target=leaf)
    OT.moments(tr, pos, gam)
    u, J = OT.evaluate(tr, pos, gam, sig, kernel="winckelmans")
    S = np.einsum("tij,tj->ti", J, gam)
    if leaf == 64:
        counts = np.asarray(tr["levels"][-1]["end"]) - np.asarray(tr["levels"][-1]["start"])
        assert counts.max() > 64
    gu, _, _ = _tree(_capi.PAIR_VELOCITY, "winckelmans", pos, gam, sig, cuda, leaf)
    gs, _, _ = _tree(_capi.PAIR_STRETCH, "winckelmans", pos, gam, sig, cuda, leaf, tg=gam)
    eu, es = rel_err(gu, u), rel_err(gs, S)
    print(f"factored loop vs oracle: velocity {eu:.2e}, stretching {es:.2e}")
    assert eu < 4e-6 and es < 4e-6


@pytest.mark.parametrize("n,leaf", [(3000, 16), (12000, 64)])
def test_paired_gaussian_vorticity_matches_oracle_algorithm(cuda, n, leaf):
    """The Gaussian-erf vorticity sweep (the Pedrizzetti relaxation's) in its
    paired loop -- erf from Abramowitz & Stegun 7.1.26 sharing the core's
    exponential, the series below rho^2 = 0.25 -- with cores 1.3 x the particle
    spacing, so that every target's self pair and its close neighbours take
    the series, against the oracle's FP64 restatement of the same treecode.
    The difference is the FP32 arithmetic and the rational erf (both well
    under the bar of the other sweeps' oracle test)."""
    pos, gam, sig = _factored_case(n=n, leaf=leaf)
    tr = OT.build(pos, theta=0.5, leaf_target=leaf)
    OT.moments(tr, pos, gam)
    _, J = OT.evaluate(tr, pos, gam, sig, kernel="gaussianerf")
    w = np.stack([J[:, 2, 1] - J[:, 1, 2], J[:, 0, 2] - J[:, 2, 0], J[:, 1, 0] - J[:, 0, 1]], 1)
    gw, _, _ = _tree(_capi.PAIR_VORTICITY, "gaussianerf", pos, gam, sig, cuda, leaf)
    e = rel_err(gw, w)
    print(f"paired Gaussian-erf vorticity vs oracle: {e:.2e}")
    assert e < 2e-5
    assert _capi.status_read_and_clear() == 0


@pytest.mark.parametrize("mode", ["velocity", "stretch"])
def test_factored_near_field_with_fp64_far_field(cuda, mode):
    """Every far pair sent to the FP64 fallback (judge tolerance ~ 0), so only
    the factored FP32 near field differs from the FP64 direct sum (5.7e-7 /
    3.5e-7 measured for velocity / stretching)."""
    pos, gam, sig = _factored_case(2500, 16, 51)
    n = pos.shape[0]
    m = _capi.PAIR_VELOCITY if mode == "velocity" else _capi.PAIR_STRETCH
    P, G, S = _dev(pos, cuda), _dev(gam, cuda), _dev(sig, cuda)
    tg = G if mode == "stretch" else None
    ref, _ = K.particle_pairs(m, P, tg, P, G, S, "winckelmans", "f64")
    ts = TreeSweeper(theta=0.5, leaf_target=16)
    ts.set_far_field("m2l")
    ts.set_validation(samples=65536, tol=1e-30)
    out = torch.empty((n, 3), dtype=torch.float64, device=cuda)
    stats = ts.sweep(m, "winckelmans", P, G, S, n, out, tgt_gamma=tg, check=True)
    assert ts.last_validation()["fallback"] == int(stats[4]) > 0
    e = rel_err(out.cpu().numpy(), ref.cpu().numpy())
    print(f"factored near field, {mode}: {e:.2e} of the FP64 direct sum")
    assert e < 4e-6
    assert _capi.status_read_and_clear() == 0
