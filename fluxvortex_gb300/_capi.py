"""ctypes binding of the fluxvortex_gb300 C ABI (include/fluxvortex_gb300.h).

The shared library is the product: every public function of this package
calls into it.  There is no CPU fallback; if the library is missing, loading
fails with an error that says how to build it.
"""
from __future__ import annotations

import ctypes
import os
import threading

from . import build as _build

P = ctypes.c_void_p
I64 = ctypes.c_int64
I32 = ctypes.c_int
D = ctypes.c_double
F = ctypes.c_float
SZ = ctypes.c_size_t

FVX_OK, FVX_ERR_ARG, FVX_ERR_CUDA, FVX_ERR_CAPACITY, FVX_ERR_TIMEOUT, FVX_ERR_SCRATCH = range(6)
LEGS_RING, LEGS_CHORDWISE, LEGS_HORSESHOE = 0, 1, 2
KERNEL_GAUSSIANERF, KERNEL_WINCKELMANS = 0, 1
KERNELS = {"gaussianerf": KERNEL_GAUSSIANERF, "winckelmans": KERNEL_WINCKELMANS}
PREC_F64, PREC_F32C = 0, 1
PRECISIONS = {"f64": PREC_F64, "fp64": PREC_F64, "f32c": PREC_F32C, "fp32c": PREC_F32C}
PAIR_VELOCITY, PAIR_STRETCH, PAIR_VELOCITY_STRETCH, PAIR_JACOBIAN, PAIR_VORTICITY = range(5)
FAR_M2P, FAR_M2L, FAR_LEARNED = range(3)

# name -> (restype, argtypes); mirrors include/fluxvortex_gb300.h
SIGNATURES = {
    "fvx_version": (ctypes.c_char_p, []),
    "fvx_last_error": (ctypes.c_char_p, []),
    "fvx_launch_count": (ctypes.c_ulonglong, []),
    "fvx_status_read_and_clear": (I32, [P, P]),
    "fvx_segments_collapsed_scratch_bytes": (SZ, [I64, I64, I32]),
    "fvx_segments_collapsed": (I32, [P, I64, P, P, P, P, P, P, P, D, I64, I32, P, P, P, SZ, P]),
    "fvx_segments_collapsed_noalloc": (I32, [P, I64, P, P, P, P, P, P, P, D, I64, I32, P, P, P]),
    "fvx_segments_expanded": (I32, [P, I64, P, P, P, P, P, P, P, D, I64, I32, P, P, P]),
    "fvx_context_create": (I32, [I32, P]),
    "fvx_context_destroy": (None, [P]),
    "fvx_host_segments_collapsed": (I32, [P, P, I64, P, P, P, P, P, P, P, D, I64, I32, P, P]),
    "fvx_host_segments_expanded": (I32, [P, P, I64, P, P, P, P, P, P, P, D, I64, I32, P, P]),
    "fvx_particle_pairs_scratch_bytes": (SZ, [I32, I32, I64, I64]),
    "fvx_particle_pairs": (I32, [I32, I32, I32, P, P, I64, P, P, P, I64, P, P, P, SZ, P]),
    "fvx_host_particle_pairs": (I32, [P, I32, I32, I32, P, P, I64, P, P, P, I64, P, P]),
    "fvx_vpm_stage_position": (I32, [I64, D, D, D, P, P, P, P, P, P]),
    "fvx_vpm_stage_strength": (I32, [I64, D, D, D, D, P, P, P, P, P, P]),
    "fvx_vpm_finalize": (I32, [I64, D, P, P, P, P]),
    "fvx_vpm_relax": (I32, [I64, D, P, P, P]),
    "fvx_probe_fp32_fma": (I32, [I32, I32, P, P]),
    "fvx_tree_create": (I32, [P]),
    "fvx_tree_destroy": (None, [P]),
    "fvx_tree_sweep": (I32, [P, I32, I32, P, P, P, P, I64, D, I32, P, P, P, P]),
    "fvx_tree_last_eval_ms": (I32, [P, P]),
    "fvx_flutter_sweep": (I32, [P, P, I32, I32, I32, P]),
    "fvx_tree_set_far_field": (I32, [P, I32, P, P, D]),
    "fvx_tree_last_local_ms": (I32, [P, P]),
    "fvx_tree_set_validation": (I32, [P, I32, D]),
    "fvx_tree_hint_same_positions": (I32, [P]),
    "fvx_tree_set_list_slots": (I32, [P, I32, I32, I32]),
    "fvx_tree_last_validation": (I32, [P, P]),
    "fvx_tree_last_judge": (I32, [P, P, I32]),
    "fvx_tree_sample_pairs": (I32, [P, I32, I32, P, P, P, P, P]),
    "fvx_mlp_forward": (I32, [P, I32, P, P, P, P, P, P]),
    "fvx_mlp_gemm": (I32, [P, I32, I32, P, I32, I32, P, I32, I32, I32, I32, I32, I32, P]),
    "fvx_mlp_loss_grad": (I32, [I32, P, P, P, P, P, P, P]),
    "fvx_mlp_silu_back": (I32, [I32, I32, P, P, P, P, P]),
    "fvx_mlp_colsum": (I32, [I32, I32, P, P, P]),
    "fvx_mlp_adam": (I32, [I32, P, P, P, P, P, F, F, F, F, I32, P]),
    "fvx_tc_gemm_probe": (I32, [P, P, I32, I32, P, I32, P]),
    "fvx_vpm_population_scratch_bytes": (SZ, [I64]),
    "fvx_vpm_drop_oldest": (I32, [I64, I64, P, P, P, P, P, P, SZ, P]),
    "fvx_vpm_merge_pass": (I32, [I64, P, P, P, P, P, I32, P, D, D, I64, D, P, P, P, SZ, P]),
    "fvx_uvlm_kinematics": (I32, [I32, P, P, D, P, P]),
    "fvx_uvlm_lattice": (I32, [P, I32, P, P, P, P, P, P, P, P, P, P, P, P]),
    "fvx_uvlm_aic": (I32, [I32, I32, P, P, P, P, P, P, D, D, P, P]),
    "fvx_uvlm_rhs": (I32, [I32, P, P, P, P, P, P, D, P, P]),
    "fvx_lu_solve_batched": (I32, [I32, I32, P, P, P]),
    "fvx_lu_workspace_bytes": (I64, [I32]),
    "fvx_lu_factor_batched": (I32, [I32, I32, P, P, P]),
    "fvx_lu_solve_factored_batched": (I32, [I32, I32, P, P, P]),
    "fvx_uvlm_loads": (I32, [I32, P, P, P, P, P, P, P, P, P, P, P, D, D, D, D, P, P, P, P]),
    "fvx_uvlm_wake_rings": (I32, [I32, P, P, P, P, D, P, P, P, P, P, P, P, P]),
    "fvx_uvlm_shed": (I32, [I32, I32, P, P, P, P, P, P, P, D, P, P, P, P, P, P, P]),
    "fvx_uvlm_loads_bernoulli": (I32, [I32, P, P, P, P, P, P, P, P, P, P, D, D, D, D, P, P, P,
                                       P]),
    "fvx_uvlm_convert": (I32, [I32, I32, P, P, P, I32, D, I64, P, P, P, P, P, P]),
}



class Surfaces(ctypes.Structure):
    """FvxSurfaces: the surface layout of a panel grid (the arrays are device
    pointers; the struct itself is passed by host pointer)."""
    _fields_ = [("ns", ctypes.c_int32), ("w", ctypes.c_int32), ("col", P), ("surf", P),
                ("motion", P)]


_lock = threading.Lock()
_lib = None
_contexts: dict[int, int] = {}


class FvxError(RuntimeError):
    """A nonzero status returned by the C ABI."""

    def __init__(self, code: int, message: str):
        super().__init__(f"fluxvortex_gb300 error {code}: {message}")
        self.code = code


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Loads (building first if needed) and returns the ctypes library."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.LIB
        if not os.path.exists(path):
            if not build_if_missing:
                raise FvxError(FVX_ERR_ARG, f"{path} not built; run "
                               "`python -m fluxvortex_gb300.build`")
            _build.build()
        lib = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def check(status: int) -> None:
    if status != FVX_OK:
        msg = load().fvx_last_error().decode(errors="replace")
        raise FvxError(status, msg)


def context(device: int = 0) -> int:
    """Process-wide host-call context for `device` (created on first use)."""
    lib = load()
    with _lock:
        h = _contexts.get(device)
        if h is None:
            out = ctypes.c_void_p()
            st = lib.fvx_context_create(device, ctypes.byref(out))
            if st != FVX_OK:
                raise FvxError(st, lib.fvx_last_error().decode(errors="replace"))
            h = out.value
            _contexts[device] = h
        return h


def status_read_and_clear(stream=None) -> int:
    bits = ctypes.c_uint(0)
    check(load().fvx_status_read_and_clear(ctypes.byref(bits), stream))
    return bits.value
