"""CPU oracle of the learned far-field operator (TEST INFRASTRUCTURE ONLY).

The operator is new -- the reference evaluates every particle sweep by direct
summation (src/fluxvortex/kernel.py:69-190) and only names a tree as future
work (docs/phase0A_findings.md:33-35) -- so there is nothing of the
reference's to pin it to.  Its pins are mathematical:
  * ``local_expansion``: the exact local expansion of a set of vortex
    particles' singular Biot-Savart field about a point, written from the
    vector potential Psi_m = (1/4pi) sum a_m / |x - x_p| (u = curl Psi) with
    the derivative tensors of oracle/treecode.py; tested against the
    quadrupole far field and against a Taylor step;
  * ``m2l``: the quadrupole expansion's local expansion (multipole to local,
    second order), with the derivative tensors of 1/r from their closed form;
    tested against ``local_expansion`` of compact clusters;
  * ``forward`` / ``gradients``: the network in FP64 with the same BF16
    rounding points as the tensor-core kernels (inputs, weights, hidden
    activations; dY and dZ for the backward GEMMs), tested against central
    differences with the rounding off.
"""
from __future__ import annotations

import numpy as np

from oracle import treecode as TC

IN, HID, OUT, NFEAT, NOUT = 48, 128, 32, 35, 30
LAYERS = ((HID, IN), (HID, HID), (HID, HID), (OUT, HID))
W_OFFSETS = (0, HID * IN, HID * IN + HID * HID, HID * IN + 2 * HID * HID)
B_OFFSETS = (0, HID, 2 * HID, 3 * HID)
KC = -1.0 / (4.0 * np.pi)   # strengths are C-scaled on the device: a' = -a / 4pi
UNIQUE = ((0, 0), (0, 1), (0, 2), (1, 1), (1, 2), (2, 2))


def bf16(x):
    """Round to the nearest BF16 (ties to even), returned as float64."""
    f = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) >> 16 << 16
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


# ---- targets and features -----------------------------------------------------------
def local_expansion(x0, pos, alpha):
    """u (3), J (3,3) [i][n] = du_i/dx_n and H (3,3,3) [i][k][n] at x0 of the
    singular field of particles (pos, alpha): u_i = eps_ijm d_j Psi_m."""
    d = x0[None, :] - pos
    D1, D2, D3, _ = TC.phi_derivs(d)
    a = alpha * (1.0 / (4.0 * np.pi))
    u = np.einsum("ijm,pm,pj->i", TC.EPS, a, D1)
    J = np.einsum("ijm,pm,pjn->in", TC.EPS, a, D2)
    H = np.einsum("ijm,pm,pjkn->ikn", TC.EPS, a, D3)
    return u, J, H


def _pairings(idx):
    """Every way to pick disjoint pairs from the positions idx: (pairs, unpaired)."""
    if not idx:
        yield [], []
        return
    first, rest = idx[0], idx[1:]
    for pr, rs in _pairings(rest):
        yield pr, [first] + rs
    for i, o in enumerate(rest):
        for pr, rs in _pairings(rest[:i] + rest[i + 1:]):
            yield [(first, o)] + pr, rs


def _dfact(n):
    return 1 if n <= 0 else n * _dfact(n - 2)


def dtensor(r, p):
    """p-th derivative tensor of 1/|r| at r (3,), from the closed form
    d^p (1/r) = sum_k (-1)^(p-k) (2p-2k-1)!! r^-(2p-2k+1) sum over the ways to
    pair 2k of the p indices (Kronecker deltas) times x for the others."""
    R = np.sqrt(r @ r)
    out = np.zeros((3,) * p)
    pl = list(_pairings(list(range(p))))
    for ii in np.ndindex(*((3,) * p)):
        s = 0.0
        for prs, rest in pl:
            if any(ii[a] != ii[b] for a, b in prs):
                continue
            k = len(prs)
            term = (-1) ** (p - k) * _dfact(2 * p - 2 * k - 1) * R ** (-(2 * p - 2 * k + 1))
            for q in rest:
                term *= r[ii[q]]
            s += term
        out[ii] = s
    return out


def m2l(R, M0, M1, M2):
    """Local expansion (u, J, H) at offset R from a cell centre of the cell's
    quadrupole expansion; moments of C-scaled strengths a' = -a/4pi, so that the
    vector potential is Psi_m = -(M0_m phi - M1_ma d_a phi + 1/2 M2_mab d_ab phi),
    phi = 1/|r|.  M1 (3,3) [m][a], M2 (3,3,3) [m][a][b]."""
    D = [None] + [dtensor(np.asarray(R, np.float64), p) for p in range(1, 6)]
    P1 = -(np.einsum("m,j->mj", M0, D[1]) - np.einsum("ma,aj->mj", M1, D[2])
           + 0.5 * np.einsum("mab,abj->mj", M2, D[3]))
    P2 = -(np.einsum("m,jn->mjn", M0, D[2]) - np.einsum("ma,ajn->mjn", M1, D[3])
           + 0.5 * np.einsum("mab,abjn->mjn", M2, D[4]))
    P3 = -(np.einsum("m,jkn->mjkn", M0, D[3]) - np.einsum("ma,ajkn->mjkn", M1, D[4])
           + 0.5 * np.einsum("mab,abjkn->mjkn", M2, D[5]))
    u = np.einsum("ijm,mj->i", TC.EPS, P1)
    J = np.einsum("ijm,mjn->in", TC.EPS, P2)
    H = np.einsum("ijm,mjkn->ikn", TC.EPS, P3)
    return u, J, H


def m2l_from_features(f):
    """Normalised (u d^2/m, J d^3/m, H d^4/m) of the quadrupole expansion from
    one pair's features (unit distance along R/d)."""
    f = np.asarray(f, np.float64)
    hs = f[3]
    M1 = f[8:17].reshape(3, 3) * hs
    M2 = np.zeros((3, 3, 3))
    for m in range(3):
        for q, (j, k) in enumerate(UNIQUE):
            M2[m, j, k] = M2[m, k, j] = f[17 + 6 * m + q] * hs * hs
    return pack_expansion(*m2l(f[0:3], f[5:8], M1, M2))


def pack_expansion(u, J, H):
    out = np.zeros(OUT)
    out[0:3] = u
    out[3:12] = J.reshape(-1)
    for i in range(3):
        for q, (k, n) in enumerate(UNIQUE):
            out[12 + 6 * i + q] = H[i, k, n]
    return out


def cell_moments(center, pos, alpha):
    """C-scaled moments in the device's record layout: M0 (3), M1 (9, [m][j]),
    M2 (18, per m: xx xy xz yy yz zz)."""
    a = alpha * KC
    d = pos - center
    M0 = a.sum(0)
    M1 = np.einsum("pm,pj->mj", a, d).reshape(-1)
    M2 = np.array([[np.sum(a[:, m] * d[:, j] * d[:, k]) for (j, k) in UNIQUE]
                   for m in range(3)]).reshape(-1)
    return M0, M1, M2


def features(cT, hT, cS, hS, M0, M1, M2):
    """Inputs (48) and the output scales (m/d^2, m/d^3, m/d^4) of one pair."""
    R = cT - cS
    d = np.sqrt(R @ R)
    n2 = sum(M2[6 * m + q] ** 2 * (1.0 if j == k else 2.0)
             for m in range(3) for q, (j, k) in enumerate(UNIQUE))
    mm = np.sqrt(M0 @ M0) + np.sqrt(M1 @ M1) / hS + np.sqrt(n2) / hS ** 2
    f = np.zeros(IN)
    f[0:3] = R / d
    f[3] = hS / d
    f[4] = hT / d
    f[5:8] = M0 / mm
    f[8:17] = M1 / (mm * hS)
    f[17:35] = M2 / (mm * hS * hS)
    return f, (mm / d ** 2, mm / d ** 3, mm / d ** 4)


def learned_pairs(tree, theta_learned):
    """(leaf, level, cell) of every accepted cell with |dc|^2 > 3/4 (h_T + h_S)^2 /
    theta_learned^2, per leaf in the traversal's depth-first order."""
    k = 0.75 / (theta_learned * theta_learned)
    levels = tree["levels"]
    leaves = levels[tree["L"]]
    out = []
    for t, (_near, far) in enumerate(TC.lists(tree)):
        cT, hT = leaves["center"][t], leaves["h"]
        for (l, c) in far:
            lev = levels[l]
            dc = cT - lev["center"][c]
            if dc @ dc > k * (hT + lev["h"]) ** 2:
                out.append((t, l, c))
    return out


def pair_features(tree, pos, alpha, pairs, target_level=None):
    """Features X (k, 48) alone of the pairs (as pair_samples, without the
    exact local expansions)."""
    perm = tree["perm"]
    sp, sa = pos[perm], alpha[perm]
    leaves = tree["levels"][tree["L"] if target_level is None else target_level]
    X = np.zeros((len(pairs), IN))
    for r, (t, l, c) in enumerate(pairs):
        lev = tree["levels"][l]
        s, e = lev["start"][c], lev["end"][c]
        M0, M1, M2 = cell_moments(lev["center"][c], sp[s:e], sa[s:e])
        X[r], _ = features(leaves["center"][t], leaves["h"], lev["center"][c], lev["h"], M0, M1,
                           M2)
    return X


def pair_samples(tree, pos, alpha, pairs, target_level=None):
    """Features X (k, 48) and normalised exact targets T (k, 32) of the pairs
    (target cells at the leaf level, or at ``target_level``)."""
    perm = tree["perm"]
    sp, sa = pos[perm], alpha[perm]
    leaves = tree["levels"][tree["L"] if target_level is None else target_level]
    X = np.zeros((len(pairs), IN))
    T = np.zeros((len(pairs), OUT))
    for r, (t, l, c) in enumerate(pairs):
        lev = tree["levels"][l]
        s, e = lev["start"][c], lev["end"][c]
        cS, hS = lev["center"][c], lev["h"]
        cT, hT = leaves["center"][t], leaves["h"]
        M0, M1, M2 = cell_moments(cS, sp[s:e], sa[s:e])
        X[r], (s2, s3, s4) = features(cT, hT, cS, hS, M0, M1, M2)
        y = pack_expansion(*local_expansion(cT, sp[s:e], sa[s:e]))
        T[r, 0:3] = y[0:3] / s2
        T[r, 3:12] = y[3:12] / s3
        T[r, 12:30] = y[12:30] / s4
    return X, T


# ---- the network -------------------------------------------------------------------
def unpack(w, b):
    Ws = [np.asarray(w[o:o + r * c], np.float64).reshape(r, c)
          for (r, c), o in zip(LAYERS, W_OFFSETS)]
    bs = [np.asarray(b[o:o + r], np.float64) for (r, _), o in zip(LAYERS, B_OFFSETS)]
    return Ws, bs


def _silu(z):
    return z / (1.0 + np.exp(-z))


def _silu_grad(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward(w, b, X, rounding=True):
    """Y (rows, 32) and the cache (Zs, Hs) of the network; rounding=True rounds
    inputs, weights and hidden activations to BF16 as the kernels do."""
    rnd = bf16 if rounding else (lambda a: np.asarray(a, np.float64))
    Ws, bs = unpack(w, b)
    h = rnd(X)
    Zs, Hs = [], [h]
    for l in range(3):
        z = h @ rnd(Ws[l]).T + bs[l]
        h = rnd(_silu(z))
        Zs.append(z)
        Hs.append(h)
    Y = h @ rnd(Ws[3]).T + bs[3]
    return Y, (Zs, Hs)


def forward_inference(w, b, X):
    """Y (rows, 32) of the far field's inference form, with the kernel's BF16
    rounding points: BF16 inputs and weights, the hidden layers' weights and
    biases halved (exact), each accumulator (z/2 - b/2, FP32 sums) rounded to
    BF16, h = BF16(acc + BF16(b/2)), t = BF16(tanh h), the activation
    BF16(h + h t) = SiLU(z) in one rounding; output layer BF16 weights, FP32
    sums plus the bias.  The kernel's tanh is the hardware approximation, so
    activations may differ by a BF16 unit in the last place."""
    Ws, bs = unpack(w, b)
    h = bf16(X)
    for l in range(3):
        acc = bf16(h @ (0.5 * bf16(Ws[l])).T)
        hh = bf16(acc + bf16(0.5 * bs[l]))
        t = bf16(np.tanh(hh))
        h = bf16(hh + hh * t)
    return h @ bf16(Ws[3]).T + bs[3]


def gradients(w, b, X, T, rounding=True):
    """Loss sum over rows and the 30 used outputs of (Y - T)^2, and the packed
    gradients (gw, gb) of the mean loss sum / (rows * 30)."""
    rnd = bf16 if rounding else (lambda a: np.asarray(a, np.float64))
    Ws, bs = unpack(w, b)
    Y, (Zs, Hs) = forward(w, b, X, rounding)
    rows = X.shape[0]
    E = np.zeros_like(Y)
    E[:, :NOUT] = Y[:, :NOUT] - T[:, :NOUT]
    loss = float((E ** 2).sum())
    dY = 2.0 * E / (rows * NOUT)
    gw = np.zeros(sum(r * c for r, c in LAYERS))
    gb = np.zeros(sum(r for r, _ in LAYERS))
    g = rnd(dY)
    gw[W_OFFSETS[3]:W_OFFSETS[3] + OUT * HID] = (g.T @ Hs[3]).reshape(-1)
    gb[B_OFFSETS[3]:B_OFFSETS[3] + OUT] = dY.sum(0)
    dH = g @ rnd(Ws[3])
    for l in (2, 1, 0):
        dZ = dH * _silu_grad(Zs[l])
        gb[B_OFFSETS[l]:B_OFFSETS[l] + HID] = dZ.sum(0)
        gz = rnd(dZ)
        r, c = LAYERS[l]
        gw[W_OFFSETS[l]:W_OFFSETS[l] + r * c] = (gz.T @ Hs[l]).reshape(-1)
        dH = gz @ rnd(Ws[l])
    return loss, gw, gb
