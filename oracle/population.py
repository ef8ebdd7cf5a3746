"""CPU oracle of particle population control (TEST INFRASTRUCTURE ONLY).

A NumPy restatement of the population control of the reference's flapping
adapter (newton_pc/adapters/flap.py of the FLUXVortex project):

- ``drop_oldest`` (flap.py:469-473): beyond ``keep`` particles the oldest --
  the front of the arrays, conversion appends at the back -- are removed.
- ``merge_pass`` (flap.py:478-563): one pass of pairwise moment-conserving
  merging judged at the wing reference points.  Candidates are the particles
  but the newest ``protect``, or with ``protect_dist`` those farther than it
  from the mean of the reference points; nothing happens while there are
  fewer than 2 ``protect`` particles (or fewer than 4 candidates in the
  distance form).  Each candidate gets the cell key floor(x / s) with
  s = 0.1 + 0.15 |x - c_wing|; in the stable lexicographic order of the keys
  (x first) consecutive candidates with equal keys pair greedily from the
  left when a1 . a2 > 0.  A pair becomes a = a1 + a2 at the |a|-weighted
  centroid (+1e-30 in the weight sum) with sigma = max, accepted when the
  largest change of the velocity it induces at the reference points
  (core g = rho^3 / (rho^2 + 1)^1.5, v = g / (4 pi d^3) (a x r),
  d = |r| + 1e-30) is below eps |V_inf|.  The merged particle replaces the
  first of the pair, the second is removed, survivors keep their order.

Pinned by tests/golden/population_merge.npz, made by running the reference's
own merge pass (tests/golden/make_golden.py).  Ages are not tracked by the
reference; here a merged particle keeps the age of the first of its pair.
"""
from __future__ import annotations

import numpy as np


def drop_oldest(pos, alpha, sigma, age, keep):
    n = pos.shape[0]
    if n <= keep:
        return pos, alpha, sigma, age
    d = n - keep
    return pos[d:], alpha[d:], sigma[d:], age[d:]


def _induced(R, X, A, S):
    """(R, M, 3) velocities at points R of particles (X, A, S)."""
    r = R[:, None, :] - X[None, :, :]
    d = np.linalg.norm(r, axis=-1) + 1e-30
    rho = d / S[None, :]
    g = rho ** 3 / (rho ** 2 + 1.0) ** 1.5
    return (g / (4 * np.pi * d ** 3))[..., None] * np.cross(A[None], r)


def merge_pass(pos, alpha, sigma, age, ref_pts, speed, eps=1e-3, protect=64, protect_dist=None):
    """Returns (pos, alpha, sigma, age, n_merged)."""
    n = pos.shape[0]
    if n < 2 * protect:
        return pos, alpha, sigma, age, 0
    c = ref_pts.mean(axis=0)
    if protect_dist:
        idx = np.flatnonzero(np.linalg.norm(pos - c, axis=1) > protect_dist)
        if idx.size < 4:
            return pos, alpha, sigma, age, 0
    else:
        idx = np.arange(n - protect)
    P, A, S = pos[idx], alpha[idx], sigma[idx]
    cell = 0.1 + 0.15 * np.linalg.norm(P - c, axis=1)
    key = np.floor(P / cell[:, None]).astype(np.int64)
    order = np.lexsort((key[:, 2], key[:, 1], key[:, 0]))
    ks = key[order]
    first, second = [], []
    taken = False
    for a in range(len(order) - 1):
        if taken:                       # order[a] is the second of the last pair
            taken = False
            continue
        if not np.array_equal(ks[a], ks[a + 1]):
            continue
        i, j = order[a], order[a + 1]
        if A[i] @ A[j] > 0.0:
            first.append(i)
            second.append(j)
            taken = True
    if not first:
        return pos, alpha, sigma, age, 0
    i, j = np.array(first), np.array(second)
    w1 = np.linalg.norm(A[i], axis=1, keepdims=True)
    w2 = np.linalg.norm(A[j], axis=1, keepdims=True)
    am = A[i] + A[j]
    xm = (w1 * P[i] + w2 * P[j]) / (w1 + w2 + 1e-30)
    sm = np.maximum(S[i], S[j])
    dv = (_induced(ref_pts, P[i], A[i], S[i]) + _induced(ref_pts, P[j], A[j], S[j])
          - _induced(ref_pts, xm, am, sm))
    ok = np.abs(dv).max(axis=(0, 2)) < eps * speed
    if not ok.any():
        return pos, alpha, sigma, age, 0
    gi, gj = idx[i[ok]], idx[j[ok]]
    pos, alpha, sigma = pos.copy(), alpha.copy(), sigma.copy()
    pos[gi], alpha[gi], sigma[gi] = xm[ok], am[ok], sm[ok]
    keep = np.ones(n, bool)
    keep[gj] = False
    return pos[keep], alpha[keep], sigma[keep], age[keep], int(ok.sum())
