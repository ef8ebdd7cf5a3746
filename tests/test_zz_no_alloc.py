"""fvx_segments_collapsed_noalloc: the collapsed ring sweep for callers that
may not allocate device memory while they run (for example a host program
that owns the GPU memory budget and passes the library only its input and
output buffers).  Called through the C ABI; its results must equal those of
fvx_segments_collapsed with a caller-provided scratch buffer, on two calls in
a row (the built-in scratch keeps the previous call's contents).

This file is named to be collected last, so a run that stops at the first
failure has already run every other test."""
import ctypes

import numpy as np
import pytest

from fluxvortex_gb300 import _capi
from tests.conftest import rel_err

pytestmark = pytest.mark.gpu
TOL = 1e-12
CAPACITY = 1 << 20   # the entry point's documented scratch limit, bytes


def _inputs(torch, dev, N, M, seed):
    rng = np.random.default_rng(seed)
    t = lambda a: torch.as_tensor(a, dtype=torch.float64, device=dev).contiguous()  # noqa: E731
    P = t(rng.standard_normal((N, 3)) * 2)
    V = [t(rng.standard_normal((M, 3)) * 2) for _ in range(4)]
    s = t(rng.standard_normal(M))
    rc = t(np.full(M, 0.03))
    ages = t(rng.uniform(0, 1, M))
    return P, V, s, rc, ages


def _with_scratch(lib, torch, dev, P, V, s, rc, ages, nu):
    N, M = P.shape[0], s.shape[0]
    out = torch.empty((N, 3), dtype=torch.float64, device=dev)
    cnt = torch.zeros(4, dtype=torch.int64, device=dev)
    nbytes = lib.fvx_segments_collapsed_scratch_bytes(N, M, _capi.LEGS_RING)
    scratch = torch.empty(max(nbytes, 1), dtype=torch.uint8, device=dev)
    _capi.check(lib.fvx_segments_collapsed(
        P.data_ptr(), N, *[v.data_ptr() for v in V], s.data_ptr(), rc.data_ptr(),
        ages.data_ptr(), nu, M, _capi.LEGS_RING, out.data_ptr(), cnt.data_ptr(),
        scratch.data_ptr(), nbytes, torch.cuda.current_stream(dev).cuda_stream))
    return out, cnt, nbytes


def _no_alloc(lib, torch, dev, P, V, s, rc, ages, nu):
    N, M = P.shape[0], s.shape[0]
    out = torch.full((N, 3), float("nan"), dtype=torch.float64, device=dev)
    cnt = torch.zeros(4, dtype=torch.int64, device=dev)
    st = lib.fvx_segments_collapsed_noalloc(
        P.data_ptr(), N, *[v.data_ptr() for v in V], s.data_ptr(), rc.data_ptr(),
        ages.data_ptr(), nu, M, _capi.LEGS_RING, out.data_ptr(), cnt.data_ptr(),
        torch.cuda.current_stream(dev).cuda_stream)
    return st, out, cnt


@pytest.mark.parametrize("N,M", [(126, 756), (500, 2000), (2000, 5000)])
def test_no_alloc_matches_scratch_entry_on_two_calls(cuda, N, M):
    import torch
    lib = _capi.load()
    P, V, s, rc, ages = _inputs(torch, cuda, N, M, seed=N + M)
    ref, ref_cnt, nbytes = _with_scratch(lib, torch, cuda, P, V, s, rc, ages, 1.5e-5)
    assert 0 < nbytes <= CAPACITY          # these sizes do use the scratch
    for call in range(2):
        st, out, cnt = _no_alloc(lib, torch, cuda, P, V, s, rc, ages, 1.5e-5)
        assert st == _capi.FVX_OK, lib.fvx_last_error()
        torch.cuda.synchronize()
        assert rel_err(out.cpu().numpy(), ref.cpu().numpy()) < TOL, f"call {call}"
        assert torch.equal(cnt, ref_cnt)


def _oversize_points(lib, M):
    """A target count whose partial sums exceed the limit on this device, or
    None.  The scratch is 24 bytes x points x splits, and the split count
    depends on the SM count, so every launch width is tried (host-side query,
    128 points per CTA, up to the width at which one split fills the GPU)."""
    for gx in range(1, 4097):
        n = 128 * gx
        nb = lib.fvx_segments_collapsed_scratch_bytes(n, M, _capi.LEGS_RING)
        if nb > CAPACITY:
            return n
        if nb == 0:          # one split already fills the GPU: no scratch beyond here
            return None
    return None


def test_no_alloc_rejects_problems_beyond_its_scratch(cuda):
    import torch
    lib = _capi.load()
    M = 200000
    N = _oversize_points(lib, M)
    if N is None:
        pytest.skip("no problem size needs more than the fixed scratch on this device")
    P, V, s, rc, ages = _inputs(torch, cuda, N, M, seed=1)
    st, out, _ = _no_alloc(lib, torch, cuda, P, V, s, rc, ages, 0.0)
    assert st == _capi.FVX_ERR_CAPACITY
    msg = lib.fvx_last_error().decode()
    assert "scratch" in msg and "fvx_segments_collapsed" in msg
    torch.cuda.synchronize()
    assert torch.isnan(out).all()          # nothing was launched


def test_no_alloc_reports_bad_arguments_before_capacity(cuda):
    import torch
    lib = _capi.load()
    M = 200000
    N = _oversize_points(lib, M) or 126
    P, V, s, rc, ages = _inputs(torch, cuda, N, M, seed=2)
    out = torch.full((N, 3), float("nan"), dtype=torch.float64, device=cuda)
    st = lib.fvx_segments_collapsed_noalloc(
        P.data_ptr(), N, *[v.data_ptr() for v in V], s.data_ptr(), rc.data_ptr(),
        ages.data_ptr(), 0.0, M, 7, out.data_ptr(), None,
        torch.cuda.current_stream(cuda).cuda_stream)
    assert st == _capi.FVX_ERR_ARG
    assert "leg set" in lib.fvx_last_error().decode()
    torch.cuda.synchronize()
    assert torch.isnan(out).all()
