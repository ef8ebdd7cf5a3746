"""Host-side parameters of the cell-binned treecode grid (shared by the device
orchestration and the tests).

The root is a cube of 2^L leaves whose corner sits on the leaf grid; the leaf
size has at most three significant bits (c 2^k, c in {1, 5/4, 3/2, 7/4}), so
every cell centre at every level is an exact binary fraction: differences of
cell centres are exact in FP32, which is what keeps the FP32 near field
accurate (pair offsets are formed as exact centre differences plus small
in-cell offsets).  The leaf size is picked from the particles' bounding box so that an
occupied leaf holds about ``leaf_target`` particles when they fill the box.
"""
from __future__ import annotations

import math

import numpy as np

MAX_LEVEL = 10          # 30-bit Morton keys


def grid_params(lo, hi, n, leaf_target=64):
    lo = np.asarray(lo, dtype=np.float64)
    hi = np.asarray(hi, dtype=np.float64)
    ext = np.maximum(hi - lo, 1e-12)
    vol = float(np.prod(np.maximum(ext, ext.max() * 1e-3)))
    h_target = (vol * leaf_target / max(n, 1)) ** (1.0 / 3.0)
    # leaf size c 2^k, c in {1, 5/4, 3/2, 7/4}: the candidate nearest to h_target
    # in ratio (boundaries at the geometric means, compared squared); three
    # significant bits keep every cell centre an exact binary fraction
    m, e = math.frexp(h_target)          # h_target = m 2^e, m in [0.5, 1)
    x = 2.0 * m                          # h_target = x 2^(e-1), x in [1, 2)
    cand = (1.0, 1.25, 1.5, 1.75, 2.0)
    ci = 0
    while ci < 4 and x * x > cand[ci] * cand[ci + 1]:
        ci += 1
    h = math.ldexp(cand[ci], e - 1)
    while True:
        origin = np.floor(lo / h) * h
        L = 1
        while h * (1 << L) <= float((hi - origin).max()):
            L += 1
        if L <= MAX_LEVEL:
            break
        h *= 2.0
    return {"L": int(L), "h": float(h), "origin": origin, "size": float(h * (1 << L))}


def _spread(v):
    v = np.asarray(v, dtype=np.uint64) & np.uint64(0x3FF)
    v = (v | (v << np.uint64(16))) & np.uint64(0x030000FF)
    v = (v | (v << np.uint64(8))) & np.uint64(0x0300F00F)
    v = (v | (v << np.uint64(4))) & np.uint64(0x030C30C3)
    v = (v | (v << np.uint64(2))) & np.uint64(0x09249249)
    return v


def morton_encode(ix, iy, iz):
    """30-bit Morton key: bit 3b = x_b, 3b+1 = y_b, 3b+2 = z_b."""
    return (_spread(ix) | (_spread(iy) << np.uint64(1)) | (_spread(iz) << np.uint64(2))).astype(
        np.int64)


def _compact(v):
    v = np.asarray(v, dtype=np.uint64) & np.uint64(0x09249249)
    v = (v | (v >> np.uint64(2))) & np.uint64(0x030C30C3)
    v = (v | (v >> np.uint64(4))) & np.uint64(0x0300F00F)
    v = (v | (v >> np.uint64(8))) & np.uint64(0x030000FF)
    v = (v | (v >> np.uint64(16))) & np.uint64(0x000003FF)
    return v.astype(np.int64)


def morton_decode(key):
    key = np.asarray(key, dtype=np.uint64)
    return _compact(key), _compact(key >> np.uint64(1)), _compact(key >> np.uint64(2))
