"""CPU oracle of the cell-binned treecode (TEST INFRASTRUCTURE ONLY).

The reference evaluates every particle sweep by direct summation
(src/fluxvortex/kernel.py:69-190); its notes name a tree/FMM method as the
missing piece for large wakes (docs/phase0A_findings.md:33-35).  The treecode
of fluxvortex_gb300 approximates those sweeps; this module restates its
algorithm in FP64 NumPy with explicit derivative tensors, so that the CUDA
kernels (which use factored contractions in FP32) can be checked against it
separately from the approximation error (which is checked against the direct
sum).

Algorithm (shared with the device code through fluxvortex_gb300.tree_params):
  1. Grid: power-of-two root cube aligned to the leaf size h; L levels.
  2. Morton key of each particle's leaf; stable sort by key.
  3. Cells at every level = runs of equal key >> 3 (L - l) in sorted order;
     geometric centres; radius r = max |x - c| over the cell's particles.
  4. Moments about the centre: M0 = sum a, M1_mj = sum a_m d_j,
     M2_mjk = sum a_m d_j d_k (d = x - c).
  5. Interaction lists per target leaf T (depth first from the root, children
     in key order): a cell S with |c_T - c_S| > (r_T + r_S) / theta is far,
     r = sqrt(3)/2 h the cell's half diagonal (compared squared:
     |dc|^2 > 3/4 (h_T + h_S)^2 / theta^2, exact in binary arithmetic, so the
     device and this oracle take identical decisions); otherwise a leaf is near
     and an inner cell is opened.
  6. Near leaves: direct pair sums with the regularised core.  Far cells: the
     quadrupole expansion of the vector potential Psi_m = (1/4pi) sum a_m / |x - x_s|
     (singular kernel; the cores are negligible beyond the acceptance
     distance): u = curl Psi, J_in = eps_ijm d_n d_j Psi_m.
  7. ``dual_lists``: the two-level lists of the local-expansion far field
     (cells shared by a parent's leaves, each leaf's own cells, near leaves),
     whose partition of the sources is tested here and whose counts pin the
     device traversal.  ``dual_lists_two_phase`` builds the same sets the way
     the device does (a walk once per parent, then each parent's residual
     cells against its leaves); a CPU test checks the two constructions agree.
"""
from __future__ import annotations

import numpy as np

from fluxvortex_gb300.tree_params import grid_params, morton_encode, morton_decode
from oracle import oracle as O

INV4PI = 1.0 / (4.0 * np.pi)


def build(pos, theta=0.5, leaf_target=64):
    pos = np.asarray(pos, dtype=np.float64)
    lo, hi = pos.min(axis=0), pos.max(axis=0)
    g = grid_params(lo, hi, pos.shape[0], leaf_target)
    L, h, origin = g["L"], g["h"], g["origin"]
    ijk = np.floor((pos - origin) * (1.0 / h)).astype(np.int64)
    ijk = np.clip(ijk, 0, (1 << L) - 1)
    keys = morton_encode(ijk[:, 0], ijk[:, 1], ijk[:, 2])
    perm = np.argsort(keys, kind="stable")
    skeys = keys[perm]
    levels = []
    for l in range(L + 1):
        kl = skeys >> (3 * (L - l))
        starts = np.flatnonzero(np.r_[True, kl[1:] != kl[:-1]])
        ends = np.r_[starts[1:], len(kl)]
        ck = kl[starts]
        ix, iy, iz = morton_decode(ck)
        hl = h * (1 << (L - l))
        center = origin + (np.stack([ix, iy, iz], 1) + 0.5) * hl
        levels.append(dict(key=ck, start=starts, end=ends, center=center, h=hl))
    # children ranges
    for l in range(L):
        child_keys = levels[l + 1]["key"] >> 3
        levels[l]["child_lo"] = np.searchsorted(child_keys, levels[l]["key"], side="left")
        levels[l]["child_hi"] = np.searchsorted(child_keys, levels[l]["key"], side="right")
    return dict(L=L, h=h, origin=origin, perm=perm, keys=skeys, levels=levels, theta=theta)


def moments(tree, pos, alpha):
    sp = pos[tree["perm"]]
    sa = alpha[tree["perm"]]
    for lev in tree["levels"]:
        n = len(lev["start"])
        M0 = np.zeros((n, 3))
        M1 = np.zeros((n, 3, 3))
        M2 = np.zeros((n, 3, 3, 3))
        r = np.zeros(n)
        for c in range(n):
            s, e = lev["start"][c], lev["end"][c]
            d = sp[s:e] - lev["center"][c]
            a = sa[s:e]
            M0[c] = a.sum(0)
            M1[c] = np.einsum("pm,pj->mj", a, d)
            M2[c] = np.einsum("pm,pj,pk->mjk", a, d, d)
            r[c] = np.sqrt((d ** 2).sum(1)).max()
        lev.update(M0=M0, M1=M1, M2=M2, r=r)


def lists(tree):
    """(near, far) per leaf: near = leaf ids, far = (level, cell) pairs."""
    L, theta = tree["L"], tree["theta"]
    levels = tree["levels"]
    leaves = levels[L]
    out = []
    for t in range(len(leaves["start"])):
        cT, hT = leaves["center"][t], leaves["h"]
        near, far = [], []
        stack = [(0, c) for c in range(len(levels[0]["start"]) - 1, -1, -1)]
        k = 0.75 / (theta * theta)
        while stack:
            l, c = stack.pop()
            lev = levels[l]
            d2 = ((cT - lev["center"][c]) ** 2).sum()
            if d2 > k * (hT + lev["h"]) ** 2:
                far.append((l, c))
            elif l == L:
                near.append(c)
            else:
                for ch in range(lev["child_hi"][c] - 1, lev["child_lo"][c] - 1, -1):
                    stack.append((l + 1, ch))
        out.append((near, far))
    return out


def phi_derivs(r):
    """Derivative tensors D1..D4 of 1/|r| at r (..., 3), from their definitions."""
    I = np.eye(3)
    r2 = np.einsum("...c,...c->...", r, r)
    R = np.sqrt(r2)[..., None]
    i3, i5 = R ** -3, R ** -5
    i7, i9 = R ** -7, R ** -9
    rr = np.einsum("...j,...k->...jk", r, r)
    D1 = -r * i3
    D2 = 3 * rr * i5[..., None] - I * i3[..., None]
    rrr = np.einsum("...j,...k,...l->...jkl", r, r, r)
    D3 = (-15 * rrr * i7[..., None, None]
          + 3 * (np.einsum("jk,...l->...jkl", I, r) + np.einsum("jl,...k->...jkl", I, r)
                 + np.einsum("kl,...j->...jkl", I, r)) * i5[..., None, None])
    D4 = (105 * np.einsum("...jk,...lm->...jklm", rr, rr) * i9[..., None, None, None]
          - 15 * (np.einsum("jk,...lm->...jklm", I, rr) + np.einsum("jl,...km->...jklm", I, rr)
                  + np.einsum("jm,...kl->...jklm", I, rr) + np.einsum("kl,...jm->...jklm", I, rr)
                  + np.einsum("km,...jl->...jklm", I, rr) + np.einsum("lm,...jk->...jklm", I, rr))
          * i7[..., None, None, None]
          + 3 * (np.einsum("jk,lm->jklm", I, I) + np.einsum("jl,km->jklm", I, I)
                 + np.einsum("jm,kl->jklm", I, I)) * i5[..., None, None, None])
    return D1, D2, D3, D4


EPS = np.zeros((3, 3, 3))
EPS[0, 1, 2] = EPS[1, 2, 0] = EPS[2, 0, 1] = 1.0
EPS[0, 2, 1] = EPS[2, 1, 0] = EPS[1, 0, 2] = -1.0


def far_field(r, M0, M1, M2):
    """Velocity u (...,3) and gradient J (...,3,3) at offsets r = x - c (...,3)
    from one cell's moments."""
    D1, D2, D3, D4 = phi_derivs(r)
    dPsi = INV4PI * (np.einsum("m,...j->...mj", M0, D1) - np.einsum("mk,...kj->...mj", M1, D2)
                     + 0.5 * np.einsum("mkl,...klj->...mj", M2, D3))
    ddPsi = INV4PI * (np.einsum("m,...nj->...mnj", M0, D2)
                      - np.einsum("mk,...knj->...mnj", M1, D3)
                      + 0.5 * np.einsum("mkl,...klnj->...mnj", M2, D4))
    u = np.einsum("ijm,...mj->...i", EPS, dPsi)
    J = np.einsum("ijm,...mnj->...in", EPS, ddPsi)
    return u, J


def evaluate(tree, pos, alpha, sigma, tgt_gamma=None, kernel="winckelmans"):
    """Treecode velocity u (N,3), Jacobian J (N,3,3) at every particle."""
    L = tree["L"]
    perm = tree["perm"]
    sp, sa, ss = pos[perm], alpha[perm], sigma[perm]
    leaves = tree["levels"][L]
    n = pos.shape[0]
    u = np.zeros((n, 3))
    J = np.zeros((n, 3, 3))
    for t, (near, far) in enumerate(lists(tree)):
        s, e = leaves["start"][t], leaves["end"][t]
        tp = sp[s:e]
        if near:
            idx = np.concatenate([np.arange(leaves["start"][c], leaves["end"][c]) for c in near])
            u[perm[s:e]] += O.velocity_from_particles(tp, sp[idx], sa[idx], ss[idx], kernel)
            J[perm[s:e]] += O.jacobian_from_particles(tp, None, sp[idx], sa[idx], ss[idx], kernel)
        for (l, c) in far:
            lev = tree["levels"][l]
            du, dJ = far_field(tp - lev["center"][c], lev["M0"][c], lev["M1"][c], lev["M2"][c])
            u[perm[s:e]] += du
            J[perm[s:e]] += dJ
    return u, J


def dual_lists(tree):
    """Two-level interaction lists of the local-expansion far field.

    For each leaf T with parent P (level L-1): source cells A are visited depth
    first from the roots; A passing the acceptance test against P goes to P's
    list (recorded by P's first child only); a failing A larger than P is
    accepted by T when it passes against the octant of P nearest to it (so all
    of P's children decide alike), else opened; a failing A of P's size or a
    leaf is tested against T: accepted (T's list), or near if a leaf, or its
    children (leaves) are each accepted or near.  The test on a pair of cells
    of sizes h_1, h_2 is |dc|^2 > 3/4 (h_1 + h_2)^2 / theta^2.
    Returns (near, leaf_far, parent_far): per leaf lists of leaf ids and of
    (level, cell), and per parent a list of (level, cell)."""
    L, theta = tree["L"], tree["theta"]
    k = 0.75 / (theta * theta)
    levels = tree["levels"]
    leaves, parents = levels[L], levels[L - 1]
    h = leaves["h"]
    near, leaf_far = [], []
    parent_far = [[] for _ in range(len(parents["start"]))]
    pkeys = parents["key"]
    for t in range(len(leaves["start"])):
        kT = leaves["key"][t]
        p = int(np.searchsorted(pkeys, kT >> 3))
        first = parents["child_lo"][p] == t
        cT, cP = leaves["center"][t], parents["center"][p]
        nr, lf = [], []

        def accept_t(l, c):
            lev = levels[l]
            d2 = ((cT - lev["center"][c]) ** 2).sum()
            if d2 > k * (h + lev["h"]) ** 2:
                lf.append((l, c))
                return True
            if l == L:
                nr.append(c)
                return True
            return False

        stack = [(0, c) for c in range(len(levels[0]["start"]) - 1, -1, -1)]
        while stack:
            l, c = stack.pop()
            lev = levels[l]
            dc = cP - lev["center"][c]
            if (dc ** 2).sum() > k * (2 * h + lev["h"]) ** 2:
                if first:
                    parent_far[p].append((l, c))
                continue
            if l < L - 1:
                near_oct = np.maximum(np.abs(dc) - 0.5 * h, 0.0)
                if (near_oct ** 2).sum() > k * (h + lev["h"]) ** 2:
                    accept_t(l, c)
                    continue
                for ch in range(lev["child_hi"][c] - 1, lev["child_lo"][c] - 1, -1):
                    stack.append((l + 1, ch))
                continue
            if accept_t(l, c):
                continue
            for q in range(lev["child_lo"][c], lev["child_hi"][c]):
                accept_t(L, q)
        near.append(nr)
        leaf_far.append(lf)
    return near, leaf_far, parent_far


def dual_lists_two_phase(tree):
    """The same lists built the way the device builds them: (1) once per parent
    P, the walk against P alone -- a cell A passing against P goes to P's list;
    A larger than P passing against the octant of P nearest to it, or A of P's
    size or a leaf failing against P, goes to P's residual list; other cells are
    opened -- and (2) per leaf T of P, the residual cells finished against T as
    in dual_lists.  Returns (near, leaf_far, parent_far) like dual_lists (the
    order within a list may differ; the sets are the same)."""
    L, theta = tree["L"], tree["theta"]
    k = 0.75 / (theta * theta)
    levels = tree["levels"]
    leaves, parents = levels[L], levels[L - 1]
    h = leaves["h"]
    parent_far, residual = [], []
    for p in range(len(parents["start"])):
        cP = parents["center"][p]
        pf, res = [], []
        stack = [(0, c) for c in range(len(levels[0]["start"]) - 1, -1, -1)]
        while stack:
            l, c = stack.pop()
            lev = levels[l]
            dc = cP - lev["center"][c]
            if (dc ** 2).sum() > k * (2 * h + lev["h"]) ** 2:
                pf.append((l, c))
                continue
            if l < L - 1:
                near_oct = np.maximum(np.abs(dc) - 0.5 * h, 0.0)
                if (near_oct ** 2).sum() > k * (h + lev["h"]) ** 2:
                    res.append((l, c))
                    continue
                for ch in range(lev["child_hi"][c] - 1, lev["child_lo"][c] - 1, -1):
                    stack.append((l + 1, ch))
                continue
            res.append((l, c))
        parent_far.append(pf)
        residual.append(res)
    pkeys = parents["key"]
    near, leaf_far = [], []
    for t in range(len(leaves["start"])):
        p = int(np.searchsorted(pkeys, leaves["key"][t] >> 3))
        cT = leaves["center"][t]
        nr, lf = [], []

        def accept_t(l, c):
            lev = levels[l]
            d2 = ((cT - lev["center"][c]) ** 2).sum()
            if d2 > k * (h + lev["h"]) ** 2:
                lf.append((l, c))
                return True
            if l == L:
                nr.append(c)
                return True
            return False

        for (l, c) in residual[p]:
            if l < L - 1:
                accept_t(l, c)
                continue
            if accept_t(l, c):
                continue
            lev = levels[l]
            for q in range(lev["child_lo"][c], lev["child_hi"][c]):
                accept_t(L, q)
        near.append(nr)
        leaf_far.append(lf)
    return near, leaf_far, parent_far
