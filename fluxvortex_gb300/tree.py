"""Cell-binned treecode sweeps over a particle set (wrapper of fvx_tree_*).

``TreeSweeper.sweep`` evaluates a self-sweep -- every particle as a target
of every particle -- with direct FP32 pairs between near leaves and a
quadrupole multipole expansion for cells accepted by the opening test
|c_T - c_S| > (r_T + r_S) / theta (r = cell half diagonal).  theta = 0.5 and
the leaf size are the defaults of the synthetic 2^20-particle sweep case.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _capi

TREE_MODES = (_capi.PAIR_VELOCITY, _capi.PAIR_STRETCH, _capi.PAIR_VELOCITY_STRETCH,
              _capi.PAIR_VORTICITY)


class TreeSweeper:
    def __init__(self, theta=0.5, leaf_target=64):
        self.theta = float(theta)
        self.leaf_target = int(leaf_target)
        self.lib = _capi.load()
        h = ctypes.c_void_p()
        _capi.check(self.lib.fvx_tree_create(ctypes.byref(h)))
        self.handle = h.value
        self.stats = np.zeros(8, dtype=np.int64)

    def __del__(self):
        try:
            if self.handle:
                self.lib.fvx_tree_destroy(self.handle)
                self.handle = None
        except Exception:
            pass

    def sweep(self, mode, kernel, pos, alpha, sigma, n, out_a, out_b=None, tgt_gamma=None,
              stream=None, check=False):
        """Device tensors (FP64 AoS) in, FP64 outputs written in place."""
        st = stream if stream is not None else torch.cuda.current_stream(pos.device).cuda_stream
        stats = self.stats.ctypes.data if check else None
        _capi.check(self.lib.fvx_tree_sweep(
            self.handle, mode, _capi.KERNELS[kernel], pos.data_ptr(), alpha.data_ptr(),
            sigma.data_ptr(), None if tgt_gamma is None else tgt_gamma.data_ptr(), int(n),
            self.theta, self.leaf_target, out_a.data_ptr(),
            None if out_b is None else out_b.data_ptr(), stats, st))
        return self.stats

    def last_eval_ms(self):
        ms = ctypes.c_float(0.0)
        _capi.check(self.lib.fvx_tree_last_eval_ms(self.handle, ctypes.byref(ms)))
        return float(ms.value)
