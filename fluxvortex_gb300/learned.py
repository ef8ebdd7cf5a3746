"""Learned far-field operator of the treecode (new: the reference has no tree).

A (target leaf T, source cell S) pair accepted by the opening test is mapped
to the local expansion of S's singular Biot-Savart field about T's centre:
velocity, velocity gradient and second derivatives (30 numbers), which the
evaluation kernel applies once per target particle.  The expansion is the
analytic multipole-to-local translation of S's quadrupole plus a learned
residual: a small MLP trained on exact FP64 local expansions, i.e. on what
the truncated quadrupole misses (the part of the higher moments that the
known moments and the cell geometry predict).  The inputs are scale free --
R/d, h_S/d, h_T/d and the cell's moments M0, M1/h_S, M2/h_S^2 divided by
m = |M0| + |M1|/h_S + |M2|/h_S^2 -- and so are the outputs (u d^2/m, J d^3/m,
H d^4/m); the kernels undo the scaling.

Everything runs on the tensor cores through the C ABI:
  * inference inside the sweep (TreeSweeper.set_far_field("learned"): one
    kernel computes the features from the pair list, the analytic translation
    on the CUDA cores and the residual on the tensor cores, and accumulates the
    expansions per leaf);
  * training (``FarFieldMLP.fit``): forward with stored activations, then per
    layer the weight gradient dW = dZ^T H and the input gradient dH = dZ W as
    BF16 tcgen05 GEMMs with FP32 accumulation, SiLU backward, Adam on FP32
    master weights with a BF16 copy for the kernels;
  * training data (``harvest``): pairs sampled from the local-expansion lists
    of the solver's own particle fields, with targets summed directly in FP64
    over the source cell's particles; the network fits T - A (exact minus
    analytic).

Weight packing (fvx_mlp_forward): W1 128x48, W2 128x128, W3 128x128, W4 32x128
as [out][in] BF16 back to back; biases 128, 128, 128, 32 in FP32.
"""
from __future__ import annotations

import math
import os

import numpy as np
import torch

from . import _capi

IN, HID, OUT, NFEAT, NOUT = 48, 128, 32, 35, 30
LAYERS = ((HID, IN), (HID, HID), (HID, HID), (OUT, HID))
W_OFFSETS = (0, HID * IN, HID * IN + HID * HID, HID * IN + 2 * HID * HID)
B_OFFSETS = (0, HID, 2 * HID, 3 * HID)
NW = HID * IN + 2 * HID * HID + OUT * HID
NB = 3 * HID + OUT
DEFAULT_WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data",
                               "farfield_mlp.npz")


def init_weights(seed=0):
    """FP32 packed (w, b): scaled normal weights, zero biases."""
    rng = np.random.default_rng(seed)
    w = np.zeros(NW, dtype=np.float32)
    for li, ((o, i), off) in enumerate(zip(LAYERS, W_OFFSETS)):
        # the output layer starts near zero: an untrained network adds no residual
        std = 0.01 * math.sqrt(1.0 / i) if li == 3 else math.sqrt(2.0 / i)
        fan_in = NFEAT if li == 0 else i
        blk = rng.standard_normal((o, i)) * std * math.sqrt(i / fan_in)
        if li == 0:
            blk[:, NFEAT:] = 0.0
        w[off:off + o * i] = blk.reshape(-1)
    return w, np.zeros(NB, dtype=np.float32)


class FarFieldMLP:
    """Device-resident weights, Adam state and training buffers."""

    def __init__(self, w=None, b=None, device="cuda", seed=0):
        if w is None:
            w, b = init_weights(seed)
        self.device = torch.device(device)
        self.w32 = torch.as_tensor(np.asarray(w, np.float32), device=self.device).contiguous()
        self.b = torch.as_tensor(np.asarray(b, np.float32), device=self.device).contiguous()
        assert self.w32.numel() == NW and self.b.numel() == NB
        self.wb = self.w32.to(torch.bfloat16)
        self.mw = torch.zeros_like(self.w32)
        self.vw = torch.zeros_like(self.w32)
        self.mb = torch.zeros_like(self.b)
        self.vb = torch.zeros_like(self.b)
        self.gw = torch.zeros_like(self.w32)
        self.gb = torch.zeros_like(self.b)
        self.step_count = 0
        self.lib = _capi.load()
        self._bufs = {}
        self.meta = {}

    # ---- persistence ---------------------------------------------------------------
    @classmethod
    def load(cls, path=DEFAULT_WEIGHTS, device="cuda"):
        z = np.load(path)
        m = cls(z["w"], z["b"], device=device)
        m.meta = {k: z[k].item() if z[k].ndim == 0 else z[k] for k in z.files
                  if k not in ("w", "b")}
        return m

    def save(self, path, **meta):
        os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
        np.savez(path, w=self.w32.cpu().numpy(), b=self.b.cpu().numpy(), **meta)

    def weights_numpy(self):
        """(BF16-rounded weights as FP32, FP32 biases) as the kernels see them."""
        return self.wb.float().cpu().numpy(), self.b.cpu().numpy()

    # ---- forward -----------------------------------------------------------------
    def _stream(self):
        return torch.cuda.current_stream(self.device).cuda_stream

    def forward(self, X, store=False):
        """X (rows, 48) BF16 -> Y (rows, 32) FP32; store=True also returns the
        pre-activations Z (3, rows, 128) FP32 and activations H (3, rows, 128) BF16."""
        rows = X.shape[0]
        assert X.dtype == torch.bfloat16 and X.shape[1] == IN and X.is_contiguous()
        Y = torch.empty((rows, OUT), dtype=torch.float32, device=self.device)
        Z = Hs = None
        if store:
            Z = torch.empty((3, rows, HID), dtype=torch.float32, device=self.device)
            Hs = torch.empty((3, rows, HID), dtype=torch.bfloat16, device=self.device)
        _capi.check(self.lib.fvx_mlp_forward(
            X.data_ptr(), rows, self.wb.data_ptr(), self.b.data_ptr(), Y.data_ptr(),
            None if Z is None else Z.data_ptr(), None if Hs is None else Hs.data_ptr(),
            self._stream()))
        return (Y, Z, Hs) if store else Y

    # ---- training ----------------------------------------------------------------
    def _gemm(self, A, lda, tA, B, ldb, tB, C, ldc, M, N, K, split_k, accumulate):
        _capi.check(self.lib.fvx_mlp_gemm(A, lda, tA, B, ldb, tB, C, ldc, M, N, K, split_k,
                                          accumulate, self._stream()))

    def _buffers(self, rows):
        bufs = self._bufs.get(rows)
        if bufs is None:
            dev = self.device
            bufs = dict(
                dY=torch.empty((rows, OUT), dtype=torch.bfloat16, device=dev),
                dY32=torch.empty((rows, OUT), dtype=torch.float32, device=dev),
                dH=torch.empty((rows, HID), dtype=torch.float32, device=dev),
                dZ=torch.empty((rows, HID), dtype=torch.bfloat16, device=dev),
                loss=torch.zeros(1, dtype=torch.float32, device=dev))
            self._bufs = {rows: bufs}
        return bufs

    def gradients(self, X, T, weights=None):
        """Loss sum(w_r (Y - T)^2) over the 30 used outputs (device scalar; w_r = 1
        without row weights) and the gradients of the mean loss into self.gw /
        self.gb."""
        rows = X.shape[0]
        Y, Z, Hs = self.forward(X, store=True)
        bf = self._buffers(rows)
        self.gw.zero_()
        self.gb.zero_()
        bf["loss"].zero_()
        st = self._stream()
        lib = self.lib
        _capi.check(lib.fvx_mlp_loss_grad(rows, Y.data_ptr(), T.data_ptr(),
                                          None if weights is None else weights.data_ptr(),
                                          bf["dY"].data_ptr(), bf["dY32"].data_ptr(),
                                          bf["loss"].data_ptr(), st))
        split = max(1, rows // 1024)
        gw, wb = self.gw.data_ptr(), self.wb.data_ptr()
        es_w, es_b = self.gw.element_size(), self.wb.element_size()
        # output layer
        self._gemm(bf["dY"].data_ptr(), OUT, 1, Hs[2].data_ptr(), HID, 1,
                   gw + W_OFFSETS[3] * es_w, HID, OUT, HID, rows, split, 1)
        _capi.check(lib.fvx_mlp_colsum(rows, OUT, bf["dY32"].data_ptr(),
                                       self.gb.data_ptr() + B_OFFSETS[3] * 4, st))
        self._gemm(bf["dY"].data_ptr(), OUT, 0, wb + W_OFFSETS[3] * es_b, HID, 1,
                   bf["dH"].data_ptr(), HID, rows, HID, OUT, 1, 0)
        # hidden layers, last to first
        for l in (2, 1, 0):
            n_in = HID if l > 0 else IN
            _capi.check(lib.fvx_mlp_silu_back(rows, HID, bf["dH"].data_ptr(), Z[l].data_ptr(),
                                              bf["dZ"].data_ptr(),
                                              self.gb.data_ptr() + B_OFFSETS[l] * 4, st))
            inp = Hs[l - 1].data_ptr() if l > 0 else X.data_ptr()
            self._gemm(bf["dZ"].data_ptr(), HID, 1, inp, n_in, 1, gw + W_OFFSETS[l] * es_w,
                       n_in, HID, n_in, rows, split, 1)
            if l > 0:
                self._gemm(bf["dZ"].data_ptr(), HID, 0, wb + W_OFFSETS[l] * es_b, n_in, 1,
                           bf["dH"].data_ptr(), HID, rows, HID, HID, 1, 0)
        return bf["loss"], Y

    def adam(self, lr, b1=0.9, b2=0.999, eps=1e-8):
        self.step_count += 1
        st = self._stream()
        _capi.check(self.lib.fvx_mlp_adam(NW, self.w32.data_ptr(), self.gw.data_ptr(),
                                          self.mw.data_ptr(), self.vw.data_ptr(),
                                          self.wb.data_ptr(), lr, b1, b2, eps, self.step_count,
                                          st))
        _capi.check(self.lib.fvx_mlp_adam(NB, self.b.data_ptr(), self.gb.data_ptr(),
                                          self.mb.data_ptr(), self.vb.data_ptr(), None, lr, b1,
                                          b2, eps, self.step_count, st))

    def fit(self, X, T, steps=2000, batch=8192, lr=2e-3, lr_final=2e-5, seed=0, log_every=0,
            weights=None):
        """Adam over random minibatches of (X, T) (optional per-row loss weights);
        cosine learning-rate decay.  Returns the mean-square losses at the
        logging points."""
        n = X.shape[0]
        g = torch.Generator(device=self.device)
        g.manual_seed(seed)
        batch = min(batch, n)
        hist = []
        for it in range(steps):
            idx = torch.randint(0, n, (batch,), device=self.device, generator=g)
            loss, _ = self.gradients(X[idx].contiguous(), T[idx].contiguous(),
                                     None if weights is None else weights[idx].contiguous())
            c = 0.5 * (1.0 + math.cos(math.pi * it / max(1, steps - 1)))
            self.adam(lr_final + (lr - lr_final) * c)
            if log_every and (it % log_every == 0 or it == steps - 1):
                hist.append((it, float(loss.item()) / (batch * NOUT)))
        return hist

    def errors(self, X, T, A):
        """Per-row relative error |A + Y - T| / |T| over the 30 used outputs
        (A: the analytic translation, T: the exact expansion)."""
        Y = self.forward(X)
        d = (A[:, :NOUT] + Y[:, :NOUT] - T[:, :NOUT]).norm(dim=1)
        return d / T[:, :NOUT].norm(dim=1).clamp_min(1e-30)


def relative_weights(T):
    """Per-row loss weights mean(|T|^2) / |T_r|^2: the fit then minimises the
    relative error of each pair's expansion rather than the absolute one."""
    n2 = T[:, :NOUT].pow(2).sum(dim=1).clamp_min(1e-30)
    return (n2.mean() / n2).float().contiguous()


def analytic_errors(T, A):
    """Per-row relative error |A - T| / |T| of the analytic translation alone."""
    d = (A[:, :NOUT] - T[:, :NOUT]).norm(dim=1)
    return d / T[:, :NOUT].norm(dim=1).clamp_min(1e-30)


def harvest(sweeper, field_pos, field_gamma, field_sigma, n, max_pairs, theta_local=None,
            kernel="winckelmans", parent_share=0.5):
    """Training pairs from one particle field: a velocity sweep on the analytic
    local-expansion path lists the pairs (theta_local defaults to the sweeper's
    theta, i.e. every accepted cell), then up to max_pairs of them are sampled
    with FP64 targets T and the analytic translation A.  Returns (X, T, A)."""
    prev = (sweeper.far_method, sweeper._mlp, sweeper.theta_local)
    sweeper.set_far_field("m2l", theta_local=theta_local)
    out = torch.empty((n, 3), dtype=torch.float64, device=field_pos.device)
    sweeper.sweep(_capi.PAIR_VELOCITY, kernel, field_pos, field_gamma, field_sigma, n, out)
    X, T, A = sweeper.sample_pairs(max_pairs, device=field_pos.device)
    if parent_share > 0:
        # the pairs shared through parents of leaves (two-level lists), which
        # the network evaluates too
        Xp, Tp, Ap = sweeper.sample_pairs(int(max_pairs * parent_share),
                                          device=field_pos.device, parents=True)
        X, T, A = torch.cat([X, Xp]), torch.cat([T, Tp]), torch.cat([A, Ap])
    sweeper.set_far_field(prev[0], prev[1], prev[2] or None)
    return X, T, A
