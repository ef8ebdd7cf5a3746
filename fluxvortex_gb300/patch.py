"""One-line drop-in: swap PteraSoftware's Biot-Savart functions for the GB300 ones.

Usage (same as ``fluxvortex.warp_patch``, src/fluxvortex/warp_patch.py:1-11)::

    from fluxvortex_gb300.patch import patch, unpatch, benchmark
    patch()      # PteraSoftware now calls the sm_103a kernels
    ...          # run PteraSoftware simulations
    unpatch()    # restore the original functions

Semantics follow warp_patch.py:25-71: the five attributes of
``pterasoftware._aerodynamics_functions`` are replaced; the originals are
saved once; ``patch()`` and ``unpatch()`` are idempotent and print one status
line each.  It works because PteraSoftware resolves these functions through
the module at call time.  ``patch(module=...)`` targets any module object with
the same attribute names (the tests use a stand-in, since PteraSoftware is a
third-party package).
"""
from __future__ import annotations

import time

import numpy as np

from . import aerodynamics as _gpu
from .aerodynamics import PS_FUNCTION_NAMES

_originals: dict = {}
_patch_active = False
_target = None


def _default_module():
    from pterasoftware import _aerodynamics_functions as af  # third-party, optional
    return af


def _save_originals(mod):
    for name in PS_FUNCTION_NAMES:
        if hasattr(mod, name) and name not in _originals:
            _originals[name] = getattr(mod, name)


def patch(module=None):
    """Replace the module's Biot-Savart functions with the GB300 kernels."""
    global _patch_active, _target
    if _patch_active:
        return
    mod = module if module is not None else _default_module()
    if _target is not None and mod is not _target:
        _originals.clear()
    _save_originals(mod)
    for name in PS_FUNCTION_NAMES:
        setattr(mod, name, getattr(_gpu, name))
    _target = mod
    _patch_active = True
    print("[fluxvortex_gb300.patch] GPU acceleration active (GB300 sm_103a kernels)")


def unpatch():
    """Restore the original functions."""
    global _patch_active
    if not _patch_active:
        return
    for name, fn in _originals.items():
        setattr(_target, name, fn)
    _patch_active = False
    print("[fluxvortex_gb300.patch] Restored original CPU functions")


def is_active() -> bool:
    return _patch_active


def benchmark(N=500, M=2000, num_runs=5, cpu_fn=None):
    """CPU original vs GB300 on random ring-vortex inputs (warp_patch.py:75-143).

    Inputs are generated exactly as warp_patch.benchmark does (rng 42).  The
    CPU side is the saved original (PteraSoftware) or ``cpu_fn``.  Times are
    wall-clock per call including host<->device transfers."""
    rng = np.random.default_rng(42)
    points = rng.standard_normal((N, 3))
    br = rng.standard_normal((M, 3))
    fr = rng.standard_normal((M, 3))
    fl = rng.standard_normal((M, 3))
    bl = rng.standard_normal((M, 3))
    strengths = rng.standard_normal(M) * 0.5
    rc0s = np.full(M, 0.03)
    sing = np.zeros(4, dtype=np.int64)
    ages = rng.uniform(0, 1, M)
    nu = 1.5e-5
    cpu = cpu_fn or _originals.get("collapsed_velocities_from_ring_vortices")
    if cpu is None:
        raise RuntimeError("no CPU implementation: patch() first or pass cpu_fn")
    args = (points, br, fr, fl, bl, strengths, rc0s, sing, ages, nu)
    cpu(*args)
    cpu_times = []
    for _ in range(num_runs):
        sing[:] = 0
        t0 = time.perf_counter()
        cpu_result = cpu(*args)
        cpu_times.append(time.perf_counter() - t0)
    _gpu.collapsed_velocities_from_ring_vortices(*args)
    gpu_times = []
    for _ in range(num_runs):
        sing[:] = 0
        t0 = time.perf_counter()
        gpu_result = _gpu.collapsed_velocities_from_ring_vortices(*args)
        gpu_times.append(time.perf_counter() - t0)
    cpu_mean, gpu_mean = float(np.mean(cpu_times)), float(np.mean(gpu_times))
    max_err = float(np.max(np.abs(cpu_result - gpu_result)))
    rel = max_err / (float(np.max(np.abs(cpu_result))) + 1e-16)
    return {"cpu_ms": cpu_mean * 1e3, "gpu_ms": gpu_mean * 1e3, "speedup": cpu_mean / gpu_mean,
            "max_abs_error": max_err, "max_rel_error": rel}
