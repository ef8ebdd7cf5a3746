"""GPU parity of the five PS-signature Biot-Savart functions against the
golden vectors (the reference's own output) and the oracle.  Tolerance: the
spec bar of 1e-12 relative (max|d| / max|ref|, the reference's
convention, tests/test_correctness.py:53-54)."""
import numpy as np
import pytest

from fluxvortex_gb300 import aerodynamics as A
from oracle import oracle as O
from tests.conftest import rel_err

pytestmark = pytest.mark.gpu
TOL = 1e-12

NAMES = {
    "collapsed_ring": "collapsed_velocities_from_ring_vortices",
    "collapsed_ring_chordwise": "collapsed_velocities_from_ring_vortices_chordwise_segments",
    "expanded_ring": "expanded_velocities_from_ring_vortices",
    "collapsed_horseshoe": "collapsed_velocities_from_horseshoe_vortices",
    "expanded_horseshoe": "expanded_velocities_from_horseshoe_vortices",
}


def _call(mod, fname, z, counts, to=None):
    args = [z[k] for k in ("points", "br", "fr", "fl", "bl", "strengths", "r_c0s")]
    ages = z["ages"]
    if to is not None:
        args = [to(a) for a in args]
        ages = to(ages)
    fn = getattr(mod, NAMES[fname])
    if "horseshoe" in fname:
        return fn(*args, counts, float(z["nu"]))
    return fn(*args, counts, ages, float(z["nu"]))


@pytest.mark.parametrize("case", ["correctness", "edge", "benchmark_small"])
@pytest.mark.parametrize("fname", list(NAMES))
def test_golden_numpy_path(cuda, golden, case, fname):
    z = golden(f"segments_{case}.npz")
    if fname not in z:
        pytest.skip("fixture holds the collapsed ring only")
    cnt = np.zeros(4, np.int64)
    r = _call(A, fname, z, cnt)
    ref = z[fname]
    assert isinstance(r, np.ndarray) and r.shape == ref.shape and r.dtype == np.float64
    assert rel_err(r, ref) < TOL
    ocnt = np.zeros(4, np.int64)
    _call(O, fname, z, ocnt)
    assert np.array_equal(cnt, ocnt)


@pytest.mark.parametrize("fname", list(NAMES))
def test_torch_device_path(cuda, golden, fname):
    import torch
    z = golden("segments_correctness.npz")
    cnt = torch.zeros(4, dtype=torch.int64, device=cuda)
    r = _call(A, fname, z, cnt, to=lambda a: torch.as_tensor(a, device=cuda))
    assert r.is_cuda
    assert rel_err(r.cpu().numpy(), z[fname]) < TOL


def test_edge_skip_counts_match_oracle(cuda, golden):
    z = golden("segments_edge.npz")
    for fname in NAMES:
        c_gpu, c_orc = np.zeros(4, np.int64), np.zeros(4, np.int64)
        _call(A, fname, z, c_gpu)
        _call(O, fname, z, c_orc)
        assert np.array_equal(c_gpu, c_orc), (fname, c_gpu, c_orc)
        assert c_gpu.sum() > 0


def test_empty_inputs(cuda):
    e3 = np.zeros((0, 3))
    cnt = np.zeros(4, np.int64)
    r = A.collapsed_velocities_from_ring_vortices(np.ones((5, 3)), e3, e3, e3, e3, np.zeros(0),
                                                  np.zeros(0), cnt)
    assert r.shape == (5, 3) and not r.any()
    r = A.expanded_velocities_from_ring_vortices(e3, *(np.ones((4, 3)),) * 4, np.ones(4),
                                                 np.ones(4), cnt)
    assert r.shape == (0, 4, 3)
    r = A.expanded_velocities_from_horseshoe_vortices(np.ones((3, 3)), e3, e3, e3, e3,
                                                      np.zeros(0), np.zeros(0), cnt)
    assert r.shape == (3, 0, 3)


@pytest.mark.parametrize("N,M", [(1, 1), (7, 3), (126, 756), (513, 1001), (2000, 5000)])
@pytest.mark.parametrize("leg", ["ring", "chordwise", "horseshoe"])
def test_random_sizes_vs_oracle(cuda, N, M, leg):
    """Ragged sizes (odd counts exercise the non-TMA tail of each tile; small N
    with large M exercises the split + fixed-order reduction)."""
    rng = np.random.default_rng(N * 7919 + M)
    P = rng.standard_normal((N, 3)) * 3
    V = [rng.standard_normal((M, 3)) * 3 for _ in range(4)]
    s = rng.standard_normal(M)
    rc = np.full(M, 0.03)
    ages = rng.uniform(0, 1, M)
    fname = {"ring": "collapsed_velocities_from_ring_vortices",
             "chordwise": "collapsed_velocities_from_ring_vortices_chordwise_segments",
             "horseshoe": "collapsed_velocities_from_horseshoe_vortices"}[leg]
    c1, c2 = np.zeros(4, np.int64), np.zeros(4, np.int64)
    if leg == "horseshoe":
        g = getattr(A, fname)(P, *V, s, rc, c1, 1.5e-5)
        o = getattr(O, fname)(P, *V, s, rc, c2, 1.5e-5)
    else:
        g = getattr(A, fname)(P, *V, s, rc, c1, ages, 1.5e-5)
        o = getattr(O, fname)(P, *V, s, rc, c2, ages, 1.5e-5)
    assert rel_err(g, o) < TOL


def test_expanded_large_vs_oracle(cuda):
    rng = np.random.default_rng(5)
    N, M = 300, 700
    P = rng.standard_normal((N, 3))
    V = [rng.standard_normal((M, 3)) for _ in range(4)]
    s = rng.standard_normal(M)
    rc = np.full(M, 0.03)
    ages = rng.uniform(0, 1, M)
    g = A.expanded_velocities_from_ring_vortices(P, *V, s, rc, None, ages, 1e-5)
    o = O.expanded_velocities_from_ring_vortices(P, *V, s, rc, None, ages, 1e-5)
    assert rel_err(g, o) < TOL


def test_unaligned_device_inputs(cuda):
    """Views starting 8 bytes into an allocation are not 16-byte aligned: the
    kernels stage them with plain loads and still agree."""
    import torch
    rng = np.random.default_rng(11)
    N, M = 129, 257
    P = rng.standard_normal((N, 3))
    V = [rng.standard_normal((M, 3)) for _ in range(4)]
    s = rng.standard_normal(M)
    rc = np.full(M, 0.03)

    def shifted(a):
        flat = torch.zeros(a.size + 1, dtype=torch.float64, device=cuda)
        flat[1:] = torch.as_tensor(a.reshape(-1), device=cuda)
        return flat[1:].view(a.shape)

    g = A.collapsed_velocities_from_ring_vortices(shifted(P), *[shifted(v) for v in V],
                                                  shifted(s), shifted(rc), None)
    o = O.collapsed_velocities_from_ring_vortices(P, *V, s, rc, None)
    assert rel_err(g.cpu().numpy(), o) < TOL
