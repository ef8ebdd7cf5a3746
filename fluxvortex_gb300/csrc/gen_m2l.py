"""Generates fvx_m2l_tensor.cuh: the analytic multipole-to-local translation of
a cell's quadrupole expansion as straight-line FP32 code.

    python fluxvortex_gb300/csrc/gen_m2l.py          # rewrites fvx_m2l_tensor.cuh

The translation (target offset n from the cell centre, |n| = 1 in the
network's normalised units; C-scaled moments c = M0, v = M1, Q = M2) is

    T1_m[j]     = c_m D1_j   - v_ma D2_aj   + 1/2 Q_mab D3_abj
    T2_m[jn]    = c_m D2_jn  - v_ma D3_ajn  + 1/2 Q_mab D4_abjn
    T3_m[jkn]   = c_m D3_jkn - v_ma D4_ajkn + 1/2 Q_mab D5_abjkn
    u_i = -eps_ijm T1_m[j],  J_in = -eps_ijm T2_m[jn],  H_ikn = -eps_ijm T3_m[jkn]

with D_p the p-th derivative tensor of 1/r at r = n, from its closed form
d^p (1/r) = sum_k (-1)^(p-k) (2p-2k-1)!! sum over the ways to pair 2k of the
p indices (Kronecker deltas) times n for the others (|n| = 1).  Every tensor
is symmetric, so only its unique components (sorted index tuples) are formed:
the 56 monomials of n up to degree 5, the 55 unique components of D1..D5,
and per source component m the components of T1..T3 that the curl reads
(j != m).  All indices are compile-time constants: the code keeps everything
in registers.

``python_twin()`` returns the same assignments as a Python function (FP64),
which the CPU tests check against the closed form of the oracle.
"""
from __future__ import annotations

import itertools
import os

UNIQUE = ((0, 0), (0, 1), (0, 2), (1, 1), (1, 2), (2, 2))
AX = "xyz"
OUT_H = os.path.join(os.path.dirname(os.path.abspath(__file__)), "fvx_m2l_tensor.cuh")


def _pairings(idx):
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


def dpoly(idx):
    """D_p component for the index tuple idx at |n| = 1: {exponents: coefficient}."""
    p = len(idx)
    poly = {}
    for prs, rest in _pairings(list(range(p))):
        if any(idx[a] != idx[b] for a, b in prs):
            continue
        k = len(prs)
        coef = (-1) ** (p - k) * _dfact(2 * p - 2 * k - 1)
        e = [0, 0, 0]
        for q in rest:
            e[idx[q]] += 1
        poly[tuple(e)] = poly.get(tuple(e), 0) + coef
    return {e: c for e, c in poly.items() if c != 0}


def _mono(e):
    return "n_" + "".join(str(x) for x in e)


def _dname(idx):
    return f"D{len(idx)}_" + "".join(AX[i] for i in sorted(idx))


def _lit(c, lang):
    return f"{float(c)!r}f" if lang == "c" else repr(float(c))


def assignments(lang):
    """(name, expression) in evaluation order, plus the output expressions."""
    A = []
    # monomials up to degree 5, each one product from a lower one
    have = {(0, 0, 0): None}
    for deg in range(1, 6):
        for e in sorted(set(tuple(sum(1 for i in c if i == a) for a in range(3))
                            for c in itertools.combinations_with_replacement(range(3), deg))):
            for a in range(3):
                if e[a] > 0:
                    lo = list(e)
                    lo[a] -= 1
                    lo = tuple(lo)
                    src = ("nx", "ny", "nz")[a]
                    A.append((_mono(e), src if sum(lo) == 0 else f"{_mono(lo)} * {src}"))
                    have[e] = True
                    break
    # unique derivative-tensor components
    for p in range(1, 6):
        for idx in itertools.combinations_with_replacement(range(3), p):
            poly = dpoly(idx)
            terms = []
            for e, c in sorted(poly.items(), key=lambda t: -sum(t[0])):
                terms.append(f"{_lit(c, lang)} * {_mono(e)}" if sum(e) else _lit(c, lang))
            A.append((_dname(idx), " + ".join(terms)))
    out = {q: [] for q in range(30)}
    for m in range(3):
        A.append((f"c{m}", f"SRC_C({m})"))
        for a in range(3):
            A.append((f"v{m}{a}", f"SRC_M1({3 * m + a}) * hs"))
        for u, (a, b) in enumerate(UNIQUE):
            half = " * " + _lit(0.5, lang) if a == b else ""
            A.append((f"q{m}{u}", f"SRC_M2({6 * m + u}) * h2{half}"))

        def contract(rest):
            """c D_rest - v_a D_(a,rest) + sum_u qw_u D_(a,b,rest)."""
            e = f"c{m} * {_dname(rest)}"
            for a in range(3):
                e += f" - v{m}{a} * {_dname(rest + (a,))}"
            for u, (a, b) in enumerate(UNIQUE):
                e += f" + q{m}{u} * {_dname(rest + (a, b))}"
            return e

        need1, need2, need3 = set(), set(), set()
        for j in range(3):
            if j == m:
                continue
            need1.add((j,))
            for n in range(3):
                need2.add(tuple(sorted((j, n))))
            for (k, n) in UNIQUE:
                need3.add(tuple(sorted((j, k, n))))
        for t in sorted(need1) + sorted(need2) + sorted(need3):
            A.append((f"T{m}_" + "".join(AX[i] for i in t), contract(t)))
        for j in range(3):
            if j == m:
                continue
            i = 3 - m - j
            sg = 1 if (j - i + 3) % 3 == 1 else -1      # eps_ijm
            op = "-" if sg > 0 else "+"
            out[i].append(f"{op} T{m}_{AX[j]}")
            for n in range(3):
                out[3 + 3 * i + n].append(f"{op} T{m}_" + "".join(AX[x] for x in sorted((j, n))))
            for u, (k, n) in enumerate(UNIQUE):
                out[12 + 6 * i + u].append(
                    f"{op} T{m}_" + "".join(AX[x] for x in sorted((j, k, n))))
    outs = [" ".join(out[q]).lstrip("+ ") if out[q][0].startswith("+") else
            "-" + " ".join(out[q])[2:] for q in range(30)]
    return A, outs


HEADER = """// fvx_m2l_tensor.cuh -- GENERATED by gen_m2l.py (same folder); do not edit.
//
// m2l_tensor: the local expansion (u, J, H in the network's normalised output
// units; u d^2/m, J d^3/m, H d^4/m) at the target centre of a source cell's
// quadrupole expansion, unit distance along n = R/d.  The derivative tensors
// D1..D5 of 1/r at r = n are formed once (unique components of the symmetric
// tensors, |n| = 1), contracted with each source component's moments
// (T_m = c_m D - v_m.D + 1/2 Q_m:D) and combined by the curl.  Src supplies
// n(i), hs() (= h_S/d), c(m) = M0/m, m1(q) = M1/(m h_S), m2(q) = M2/(m h_S^2)
// (six unique components per m); out[q] is written once per q.
#pragma once

namespace fvx {
namespace mlp {

template <class Src, class Out>
__device__ __forceinline__ void m2l_tensor(const Src& src, Out&& out) {
  const float nx = src.n(0), ny = src.n(1), nz = src.n(2);
  const float hs = src.hs();
  const float h2 = hs * hs;
"""


def cuda_source():
    A, outs = assignments("c")
    lines = [HEADER]
    for name, e in A:
        e = (e.replace("SRC_C(", "src.c(").replace("SRC_M1(", "src.m1(")
             .replace("SRC_M2(", "src.m2("))
        lines.append(f"  const float {name} = {e};\n")
    for q, e in enumerate(outs):
        lines.append(f"  out[{q}] = {e};\n")
    lines.append("}\n\n}  // namespace mlp\n}  // namespace fvx\n")
    return "".join(lines)


def python_twin():
    """f(n (3,), c (3,), M1 (9,) = M1/(m h_S), M2 (18,) = M2/(m h_S^2), hs) -> out (30,)."""
    A, outs = assignments("py")
    body = ["def m2l_tensor(n, c, M1, M2, hs):",
            "    nx, ny, nz = float(n[0]), float(n[1]), float(n[2])",
            "    h2 = hs * hs"]
    for name, e in A:
        e = (e.replace("SRC_C(", "c[").replace("SRC_M1(", "M1[").replace("SRC_M2(", "M2[")
             .replace(")", "]"))
        body.append(f"    {name} = {e}")
    body.append("    return [" + ", ".join(f"({e})" for e in outs) + "]")
    ns = {}
    exec("\n".join(body), ns)  # noqa: S102 -- code generated above from fixed tables
    return ns["m2l_tensor"]


if __name__ == "__main__":
    with open(OUT_H, "w") as f:
        f.write(cuda_source())
    print(OUT_H)
