"""Vortex-particle Biot-Savart sweeps on the GB300 (mirror of kernel.py).

Same call signatures as ``src/fluxvortex/kernel.py:69`` and ``:119``
(``velocity_from_particles``, ``jacobian_from_particles``) plus
``velocity_and_stretching`` and ``vorticity_from_particles``, all with an
optional ``precision`` ("f64" or "f32c": FP32 pair arithmetic with
compensated accumulation).  NumPy inputs take the synchronous host path;
torch CUDA tensors take the zero-copy stream-ordered device path.

Self pairs follow kernel.py's r -> 1e-12 clamp limit.  The Gaussian-erf core
is evaluated without the cancellation of kernel.py:16-18 (series below
r/sigma = 0.5); elsewhere results agree with kernel.py to rounding.
"""
from __future__ import annotations

import numpy as np

from . import _capi

__all__ = ["velocity_from_particles", "jacobian_from_particles", "velocity_and_stretching",
           "vorticity_from_particles", "particle_pairs"]

_NCOMP = {_capi.PAIR_VELOCITY: (3, 0), _capi.PAIR_STRETCH: (3, 0),
          _capi.PAIR_VELOCITY_STRETCH: (3, 3), _capi.PAIR_JACOBIAN: (9, 0),
          _capi.PAIR_VORTICITY: (3, 0)}


def _is_cuda_tensor(x) -> bool:
    return getattr(x, "is_cuda", False) and hasattr(x, "data_ptr")


def particle_pairs(mode, tgt_pos, tgt_gamma, src_pos, src_gamma, src_sigma,
                   kernel="winckelmans", precision="f64", stream=None):
    """One all-pairs sweep; returns (out_a, out_b or None).  See the
    FVX_PAIR_* table of include/fluxvortex_gb300.h for the outputs."""
    lib = _capi.load()
    kid = _capi.KERNELS[kernel]
    pid = _capi.PRECISIONS[precision]
    na, nb = _NCOMP[mode]
    if _is_cuda_tensor(tgt_pos):
        import torch
        dev = tgt_pos.device

        def f64(x, tail):
            t = torch.as_tensor(x, device=dev, dtype=torch.float64).contiguous()
            return t.reshape((-1,) + tail) if tail else t.reshape(-1)

        t = f64(tgt_pos, (3,))
        tg = None if tgt_gamma is None else f64(tgt_gamma, (3,))
        p, g, s = f64(src_pos, (3,)), f64(src_gamma, (3,)), f64(src_sigma, ())
        M, N = t.shape[0], p.shape[0]
        a = torch.empty((M, na), device=dev, dtype=torch.float64)
        b = torch.empty((M, nb), device=dev, dtype=torch.float64) if nb else None
        st = stream if stream is not None else torch.cuda.current_stream(dev).cuda_stream
        nbytes = lib.fvx_particle_pairs_scratch_bytes(mode, pid, M, N)
        scratch = torch.empty(max(nbytes, 1), device=dev, dtype=torch.uint8)
        with torch.cuda.device(dev):
            _capi.check(lib.fvx_particle_pairs(
                mode, kid, pid, t.data_ptr(), None if tg is None else tg.data_ptr(), M,
                p.data_ptr(), g.data_ptr(), s.data_ptr(), N, a.data_ptr(),
                None if b is None else b.data_ptr(), scratch.data_ptr(), nbytes, st))
        return a, b
    t = np.ascontiguousarray(tgt_pos, dtype=np.float64).reshape(-1, 3)
    tg = None if tgt_gamma is None else np.ascontiguousarray(tgt_gamma, np.float64).reshape(-1, 3)
    p = np.ascontiguousarray(src_pos, dtype=np.float64).reshape(-1, 3)
    g = np.ascontiguousarray(src_gamma, dtype=np.float64).reshape(-1, 3)
    s = np.ascontiguousarray(src_sigma, dtype=np.float64).reshape(-1)
    if g.shape[0] != p.shape[0] or s.shape[0] != p.shape[0]:
        raise ValueError("src_pos, src_gamma and src_sigma must have the same length")
    M, N = t.shape[0], p.shape[0]
    a = np.zeros((M, na))
    b = np.zeros((M, nb)) if nb else None
    if M == 0:
        return a, b
    _capi.check(lib.fvx_host_particle_pairs(
        _capi.context(0), mode, kid, pid, t.ctypes.data, None if tg is None else tg.ctypes.data,
        M, p.ctypes.data, g.ctypes.data, s.ctypes.data, N, a.ctypes.data,
        None if b is None else b.ctypes.data))
    return a, b


def velocity_from_particles(target_points, src_pos, src_gamma, src_sigma,
                            kernel="gaussianerf", precision="f64"):
    """(M,3) velocity induced at target_points (kernel.py:69-116)."""
    u, _ = particle_pairs(_capi.PAIR_VELOCITY, target_points, None, src_pos, src_gamma,
                          src_sigma, kernel, precision)
    return u


def jacobian_from_particles(tgt_pos, tgt_gamma, src_pos, src_gamma, src_sigma,
                            kernel="gaussianerf", precision="f64"):
    """(M,3,3) velocity gradient J[t,i,j] = du_i/dx_j (kernel.py:119-190).
    tgt_gamma is unused, as in the reference."""
    J, _ = particle_pairs(_capi.PAIR_JACOBIAN, tgt_pos, None, src_pos, src_gamma, src_sigma,
                          kernel, precision)
    return J.reshape(-1, 3, 3)


def velocity_and_stretching(tgt_pos, tgt_gamma, src_pos, src_gamma, src_sigma,
                            kernel="winckelmans", precision="f64"):
    """u (M,3) and S = J . Gamma_t (M,3) from one sweep at the same state."""
    return particle_pairs(_capi.PAIR_VELOCITY_STRETCH, tgt_pos, tgt_gamma, src_pos, src_gamma,
                          src_sigma, kernel, precision)


def stretching_from_particles(tgt_pos, tgt_gamma, src_pos, src_gamma, src_sigma,
                              kernel="winckelmans", precision="f64"):
    """S = J . Gamma_t (M,3) (particles.py:148-151)."""
    S, _ = particle_pairs(_capi.PAIR_STRETCH, tgt_pos, tgt_gamma, src_pos, src_gamma, src_sigma,
                          kernel, precision)
    return S


def vorticity_from_particles(tgt_pos, src_pos, src_gamma, src_sigma, kernel="gaussianerf",
                             precision="f64"):
    """omega_i = eps_ijk J_kj (M,3), the curl used by particles.py:219-225."""
    w, _ = particle_pairs(_capi.PAIR_VORTICITY, tgt_pos, None, src_pos, src_gamma, src_sigma,
                          kernel, precision)
    return w
