"""Cell-binned treecode sweeps over a particle set (wrapper of fvx_tree_*).

``TreeSweeper.sweep`` evaluates a self-sweep -- every particle as a target
of every particle -- with direct FP32 pairs between near leaves and a
quadrupole multipole expansion for cells accepted by the opening test
|c_T - c_S| > (r_T + r_S) / theta (r = cell half diagonal).  The accepted
cells are evaluated either at every target particle ("m2p") or once per
target leaf as a local expansion ("m2l": analytic translation; "learned":
plus a tensor-core MLP residual), see ``set_far_field``.  theta = 0.5 and the
leaf size are the defaults of the synthetic 2^20-particle sweep case.
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
        self._mlp = None
        self.far_method = "m2p"
        self.theta_local = 0.0

    def __del__(self):
        try:
            if self.handle:
                self.lib.fvx_tree_destroy(self.handle)
                self.handle = None
        except Exception:
            pass

    def sweep(self, mode, kernel, pos, alpha, sigma, n, out_a, out_b=None, tgt_gamma=None,
              stream=None, check=False, same_positions=False):
        """Device tensors (FP64 AoS) in, FP64 outputs written in place.
        ``same_positions``: the positions are those of the last full build
        (the tree structure is reused; see fvx_tree_hint_same_positions)."""
        st = stream if stream is not None else torch.cuda.current_stream(pos.device).cuda_stream
        stats = self.stats.ctypes.data if check else None
        if same_positions:
            _capi.check(self.lib.fvx_tree_hint_same_positions(self.handle))
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

    # ---- far-field method ---------------------------------------------------------
    def set_far_field(self, method="m2p", mlp=None, theta_local=None):
        """"m2p": quadrupole at every target particle (default).  "m2l": the
        accepted cells with |dc|^2 > 3/4 (h_T + h_S)^2 / theta_local^2 (all of
        them for theta_local = theta, the default) go through per-leaf local
        expansions from the analytic multipole-to-local translation.
        "learned": the same plus the residual of ``mlp`` (a learned.FarFieldMLP
        whose device weights must outlive the sweeps)."""
        mid = {"m2p": _capi.FAR_M2P, "m2l": _capi.FAR_M2L, "learned": _capi.FAR_LEARNED}[method]
        th = 0.0 if mid == _capi.FAR_M2P else float(theta_local or self.theta)
        if mid == _capi.FAR_LEARNED and mlp is None:
            raise ValueError("the learned far field needs a FarFieldMLP")
        self._mlp = mlp if mid == _capi.FAR_LEARNED else None
        W = None if self._mlp is None else self._mlp.wb.data_ptr()
        b = None if self._mlp is None else self._mlp.b.data_ptr()
        _capi.check(self.lib.fvx_tree_set_far_field(self.handle, mid, W, b, th))
        self.far_method = method
        self.theta_local = th

    def set_list_slots(self, near=512, lrn=1024, par=1024):
        """Slot capacities of the one-pass two-level lists (0: always count)."""
        _capi.check(self.lib.fvx_tree_set_list_slots(self.handle, int(near), int(lrn), int(par)))

    def set_validation(self, samples=256, tol=0.1):
        """The FP64 judge of the local-expansion path for the next sweeps:
        ``samples`` pairs per judged sweep, stratified over the 16 pair classes
        (list x cell larger than target x opening-ratio bin); per class the
        network is kept, dropped, or the whole class is summed directly in FP64,
        and sampled pairs above ``tol`` are summed directly in FP64
        (fvx_tree_set_validation).  samples=0: the next sweeps are not judged
        and keep the last judged sweep's class decisions."""
        _capi.check(self.lib.fvx_tree_set_validation(self.handle, int(samples), float(tol)))

    def last_validation(self):
        """{checked, fallback, mean_err, max_err} of the last judged sweep
        (fallback: pairs summed directly in FP64, whole classes included)."""
        j = self.last_judge()
        return {"checked": j["checked"], "fallback": j["fp64_pairs"], "mean_err": j["mean_err"],
                "max_err": j["max_err"]}

    JUDGE_ACTIONS = ("network", "translation", "fp64")

    def last_judge(self):
        """The full record of the last judged sweep (fvx_tree_last_judge):
        pairs judged and repaired, pairs summed directly in FP64, mean / max
        applied error, the estimated fraction of the path's pairs left above
        the tolerance, and per class its pairs, samples, failures with and
        without the network and the action taken."""
        out = np.zeros(8 + 5 * 16, dtype=np.float64)
        _capi.check(self.lib.fvx_tree_last_judge(self.handle, out.ctypes.data, out.size))
        cls = out[8:].reshape(16, 5)
        return {"checked": int(out[0]), "repaired": int(out[1]), "fp64_pairs": int(out[2]),
                "mean_err": float(out[3]), "max_err": float(out[4]),
                "unrepaired_est": float(out[5]), "pairs": int(out[6]),
                "classes": [{"class": k, "pairs": int(c[0]), "samples": int(c[1]),
                             "fail_network": int(c[2]), "fail_translation": int(c[3]),
                             "action": self.JUDGE_ACTIONS[int(c[4])]}
                            for k, c in enumerate(cls) if c[0] > 0]}

    def last_local_ms(self):
        ms = ctypes.c_float(0.0)
        _capi.check(self.lib.fvx_tree_last_local_ms(self.handle, ctypes.byref(ms)))
        return float(ms.value)

    def sample_pairs(self, max_pairs, stream=None, device="cuda", parents=False):
        """Features X (k, 48) BF16, exact normalised targets T (k, 32) and the
        analytic translation A (k, 32) of up to max_pairs local-path pairs of the
        last sweep (evenly strided over its list): the leaves' own pairs, or with
        parents=True the pairs shared through parents of leaves."""
        X = torch.empty((max_pairs, 48), dtype=torch.bfloat16, device=device)
        T = torch.empty((max_pairs, 32), dtype=torch.float32, device=device)
        A = torch.empty((max_pairs, 32), dtype=torch.float32, device=device)
        st = stream if stream is not None else torch.cuda.current_stream(X.device).cuda_stream
        k = ctypes.c_int(0)
        _capi.check(self.lib.fvx_tree_sample_pairs(self.handle, 1 if parents else 0,
                                                    int(max_pairs), X.data_ptr(),
                                                    T.data_ptr(), A.data_ptr(), ctypes.byref(k),
                                                    st))
        return X[: k.value], T[: k.value], A[: k.value]
