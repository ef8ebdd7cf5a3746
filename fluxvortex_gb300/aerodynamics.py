"""PteraSoftware-signature Biot-Savart functions backed by the sm_103a library.

Drop-in replacements for the five functions that
``src/fluxvortex/warp_kernels.py:251-382`` provides and that
``src/fluxvortex/warp_patch.py:51-55`` swaps into
``pterasoftware._aerodynamics_functions``.  Same positional signatures, same
(N,3) / (N,M,3) float64 results, same empty-input behaviour
(``warp_kernels.py:193-194, 224-225``).

Two call forms:
  * NumPy arrays (what PteraSoftware passes): one host-to-device transfer of
    all inputs, one fused launch, one device-to-host transfer, synchronous; a
    new NumPy array is returned.
  * torch CUDA tensors: zero-copy, stream-ordered on torch's current stream;
    a new CUDA tensor is returned.

``singularity_counts`` (int64[4]) is incremented per skipped (point, leg)
pair: [0] zero-length leg (warp_kernels.py:52), [1] point at the leg start
(:72), [2] point at the leg end (:74), [3] point on the leg's line (:81).
The reference's Warp path leaves it untouched; PteraSoftware's own functions
count singular cases into it.
"""
from __future__ import annotations

import numpy as np

from . import _capi

__all__ = [
    "collapsed_velocities_from_ring_vortices",
    "collapsed_velocities_from_ring_vortices_chordwise_segments",
    "expanded_velocities_from_ring_vortices",
    "collapsed_velocities_from_horseshoe_vortices",
    "expanded_velocities_from_horseshoe_vortices",
    "PS_FUNCTION_NAMES",
]


def _is_cuda_tensor(x) -> bool:
    return getattr(x, "is_cuda", False) and hasattr(x, "data_ptr")


def _host_f64(a, shape_tail):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a.reshape((-1,) + shape_tail) if shape_tail else a.reshape(-1)


def _ptr(a):
    return None if a is None else a.ctypes.data


def _segments_host(expanded, leg_set, points, br, fr, fl, bl, strengths, r_c0s, counts, ages, nu):
    lib = _capi.load()
    P = _host_f64(points, (3,))
    C = [_host_f64(x, (3,)) for x in (br, fr, fl, bl)]
    s = _host_f64(strengths, ())
    rc = _host_f64(r_c0s, ())
    a = None if ages is None else _host_f64(ages, ())
    N, M = P.shape[0], s.shape[0]
    if any(c.shape[0] != M for c in C) or rc.shape[0] != M or (a is not None and a.shape[0] != M):
        raise ValueError("vortex arrays must all have strengths.shape[0] rows")
    out = np.empty((N, M, 3) if expanded else (N, 3), dtype=np.float64)
    cnt = np.zeros(4, dtype=np.int64)
    fn = lib.fvx_host_segments_expanded if expanded else lib.fvx_host_segments_collapsed
    _capi.check(fn(_capi.context(0), _ptr(P), N, *[_ptr(c) for c in C], _ptr(s), _ptr(rc),
                   _ptr(a), float(nu), M, leg_set, _ptr(out), _ptr(cnt)))
    _add_counts(counts, cnt)
    return out


def _add_counts(counts, cnt):
    if counts is None:
        return
    if isinstance(counts, np.ndarray) and counts.size >= 4:
        counts.reshape(-1)[:4] += cnt.astype(counts.dtype)
    elif _is_cuda_tensor(counts):
        import torch
        counts.view(-1)[:4] += torch.as_tensor(cnt, device=counts.device, dtype=counts.dtype)


def _segments_device(expanded, leg_set, points, br, fr, fl, bl, strengths, r_c0s, counts, ages, nu):
    import torch
    lib = _capi.load()
    dev = points.device

    def f64(x, tail):
        t = torch.as_tensor(x, device=dev, dtype=torch.float64).contiguous()
        return t.reshape((-1,) + tail) if tail else t.reshape(-1)

    P = f64(points, (3,))
    C = [f64(x, (3,)) for x in (br, fr, fl, bl)]
    s = f64(strengths, ())
    rc = f64(r_c0s, ())
    a = None if ages is None else f64(ages, ())
    N, M = P.shape[0], s.shape[0]
    stream = torch.cuda.current_stream(dev).cuda_stream
    out = torch.empty((N, M, 3) if expanded else (N, 3), device=dev, dtype=torch.float64)
    dcnt = torch.zeros(4, device=dev, dtype=torch.int64)
    ap = None if a is None else a.data_ptr()
    with torch.cuda.device(dev):
        if expanded:
            st = lib.fvx_segments_expanded(P.data_ptr(), N, *[c.data_ptr() for c in C],
                                           s.data_ptr(), rc.data_ptr(), ap, float(nu), M, leg_set,
                                           out.data_ptr(), dcnt.data_ptr(), stream)
        else:
            nbytes = lib.fvx_segments_collapsed_scratch_bytes(N, M, leg_set)
            scratch = torch.empty(max(nbytes, 1), device=dev, dtype=torch.uint8)
            st = lib.fvx_segments_collapsed(P.data_ptr(), N, *[c.data_ptr() for c in C],
                                            s.data_ptr(), rc.data_ptr(), ap, float(nu), M, leg_set,
                                            out.data_ptr(), dcnt.data_ptr(), scratch.data_ptr(),
                                            nbytes, stream)
    _capi.check(st)
    if counts is not None:
        if _is_cuda_tensor(counts):
            counts.view(-1)[:4] += dcnt.to(counts.dtype)
        else:
            _add_counts(counts, dcnt.cpu().numpy())
    return out


def _segments(expanded, leg_set, points, br, fr, fl, bl, strengths, r_c0s, counts, ages, nu):
    if _is_cuda_tensor(points):
        return _segments_device(expanded, leg_set, points, br, fr, fl, bl, strengths, r_c0s,
                                counts, ages, nu)
    return _segments_host(expanded, leg_set, points, br, fr, fl, bl, strengths, r_c0s, counts,
                          ages, nu)


def collapsed_velocities_from_ring_vortices(
        stackP_GP1_CgP1, stackBrrvp_GP1_CgP1, stackFrrvp_GP1_CgP1, stackFlrvp_GP1_CgP1,
        stackBlrvp_GP1_CgP1, strengths, r_c0s, singularity_counts, ages=None, nu=0.0):
    """(N,3) velocity at N points summed over M ring vortices (4 legs each).
    Replaces warp_kernels.py:251-276."""
    return _segments(False, _capi.LEGS_RING, stackP_GP1_CgP1, stackBrrvp_GP1_CgP1,
                     stackFrrvp_GP1_CgP1, stackFlrvp_GP1_CgP1, stackBlrvp_GP1_CgP1, strengths,
                     r_c0s, singularity_counts, ages, nu)


def collapsed_velocities_from_ring_vortices_chordwise_segments(
        stackP_GP1_CgP1, stackBrrvp_GP1_CgP1, stackFrrvp_GP1_CgP1, stackFlrvp_GP1_CgP1,
        stackBlrvp_GP1_CgP1, strengths, r_c0s, singularity_counts, ages=None, nu=0.0):
    """As the ring function with only the right (BR->FR) and left (FL->BL)
    legs.  Replaces warp_kernels.py:279-302."""
    return _segments(False, _capi.LEGS_CHORDWISE, stackP_GP1_CgP1, stackBrrvp_GP1_CgP1,
                     stackFrrvp_GP1_CgP1, stackFlrvp_GP1_CgP1, stackBlrvp_GP1_CgP1, strengths,
                     r_c0s, singularity_counts, ages, nu)


def expanded_velocities_from_ring_vortices(
        stackP_GP1_CgP1, stackBrrvp_GP1_CgP1, stackFrrvp_GP1_CgP1, stackFlrvp_GP1_CgP1,
        stackBlrvp_GP1_CgP1, strengths, r_c0s, singularity_counts, ages=None, nu=0.0):
    """(N,M,3) velocity of each ring vortex at each point.  Replaces
    warp_kernels.py:305-332."""
    return _segments(True, _capi.LEGS_RING, stackP_GP1_CgP1, stackBrrvp_GP1_CgP1,
                     stackFrrvp_GP1_CgP1, stackFlrvp_GP1_CgP1, stackBlrvp_GP1_CgP1, strengths,
                     r_c0s, singularity_counts, ages, nu)


def collapsed_velocities_from_horseshoe_vortices(
        stackP_GP1_CgP1, stackBrhvp_GP1_CgP1, stackFrhvp_GP1_CgP1, stackFlhvp_GP1_CgP1,
        stackBlhvp_GP1_CgP1, strengths, r_c0s, singularity_counts, nu=0.0):
    """(N,3) velocity summed over horseshoe vortices (3 legs, zero ages).
    Replaces warp_kernels.py:335-357."""
    return _segments(False, _capi.LEGS_HORSESHOE, stackP_GP1_CgP1, stackBrhvp_GP1_CgP1,
                     stackFrhvp_GP1_CgP1, stackFlhvp_GP1_CgP1, stackBlhvp_GP1_CgP1, strengths,
                     r_c0s, singularity_counts, None, nu)


def expanded_velocities_from_horseshoe_vortices(
        stackP_GP1_CgP1, stackBrhvp_GP1_CgP1, stackFrhvp_GP1_CgP1, stackFlhvp_GP1_CgP1,
        stackBlhvp_GP1_CgP1, strengths, r_c0s, singularity_counts, nu=0.0):
    """(N,M,3) velocity of each horseshoe vortex at each point.  Replaces
    warp_kernels.py:360-382."""
    return _segments(True, _capi.LEGS_HORSESHOE, stackP_GP1_CgP1, stackBrhvp_GP1_CgP1,
                     stackFrhvp_GP1_CgP1, stackFlhvp_GP1_CgP1, stackBlhvp_GP1_CgP1, strengths,
                     r_c0s, singularity_counts, None, nu)


PS_FUNCTION_NAMES = (
    "collapsed_velocities_from_ring_vortices",
    "collapsed_velocities_from_ring_vortices_chordwise_segments",
    "expanded_velocities_from_ring_vortices",
    "collapsed_velocities_from_horseshoe_vortices",
    "expanded_velocities_from_horseshoe_vortices",
)
