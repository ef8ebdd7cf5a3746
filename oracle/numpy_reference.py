"""NumPy restatement of the reference's CPU particle kernels (TEST
INFRASTRUCTURE ONLY: the timed baseline of the reference's own NumPy path).

The reference's CPU hot path for the particle sweeps is
``fluxvortex.kernel.velocity_from_particles`` and ``jacobian_from_particles``
(src/fluxvortex/kernel.py:69-116, :119-190), called by
``VortexParticleField.advect_rk3`` (src/fluxvortex/particles.py:122, :148).
That module cannot be shipped to the machine that runs the benchmark, so it
is restated here with the same algorithm and the same cost profile: FP64,
targets and sources in blocks of 512 (kernel.py:66), every block pair
evaluated with full (Bt, Bs, 3) temporaries -- offsets, squared distances,
the Winckelmans or Gaussian-erf core at r/sigma, the cross product with the
source strengths and a reduction over the sources -- on one NumPy thread.
Results are pinned to the reference's own outputs (tests/golden/
particles_kernel.npz) in tests/test_oracle_golden.py.  Nothing on the product
path imports this file.
"""
from __future__ import annotations

import math
import time

import numpy as np
from scipy.special import erf

BLOCK = 512
_C = -1.0 / (4.0 * math.pi)


def _core(rb, kernel):
    """g(r/sigma) and dg/d(r/sigma) of the two cores (kernel.py:10-56)."""
    if kernel == "winckelmans":
        q = rb * rb + 1.0
        return rb ** 3 * (rb * rb + 2.5) / q ** 2.5, 7.5 * rb * rb / q ** 3.5
    e = np.exp(-0.5 * rb * rb)
    c = math.sqrt(2.0 / math.pi)
    return erf(rb / math.sqrt(2.0)) - c * rb * e, c * rb * rb * e


def velocity_from_particles(tgt, pos, gam, sig, kernel="winckelmans"):
    """(M, 3) velocities at tgt from the particles (kernel.py:69-116)."""
    M, N = tgt.shape[0], pos.shape[0]
    U = np.zeros((M, 3))
    for i0 in range(0, M, BLOCK):
        t = tgt[i0:i0 + BLOCK]
        for j0 in range(0, N, BLOCK):
            d = t[:, None, :] - pos[None, j0:j0 + BLOCK, :]
            r = np.maximum(np.sqrt(np.sum(d * d, axis=-1)), 1e-12)
            g, _ = _core(r / sig[None, j0:j0 + BLOCK], kernel)
            cr = np.cross(d, gam[None, j0:j0 + BLOCK, :])
            U[i0:i0 + BLOCK] += np.sum((_C * g / r ** 3)[:, :, None] * cr, axis=1)
    return U


def jacobian_from_particles(tgt, pos, gam, sig, kernel="winckelmans"):
    """(M, 3, 3) velocity gradients dU_i/dx_j at tgt (kernel.py:119-190)."""
    M, N = tgt.shape[0], pos.shape[0]
    J = np.zeros((M, 3, 3))
    for i0 in range(0, M, BLOCK):
        t = tgt[i0:i0 + BLOCK]
        for j0 in range(0, N, BLOCK):
            s = slice(j0, j0 + BLOCK)
            d = t[:, None, :] - pos[None, s, :]
            r = np.sqrt(np.maximum(np.sum(d * d, axis=-1), 1e-24))
            sg = sig[None, s]
            g, dg = _core(r / sg, kernel)
            ir3 = 1.0 / r ** 3
            kg = _C * np.cross(d, gam[None, s, :]) * ir3[:, :, None]
            aux = dg / (sg * r) - 3.0 * g / r ** 2
            aux2 = _C * g * ir3
            a = gam[None, s, :]
            # the gradient of (d x a) g / r^3: the radial part and the
            # antisymmetric part of the cross product
            J[i0:i0 + BLOCK] += np.einsum("tsi,tsj->tij", aux[:, :, None] * kg, d)
            J[i0:i0 + BLOCK, 0, 1] += np.sum(aux2 * a[..., 2], axis=1)
            J[i0:i0 + BLOCK, 0, 2] -= np.sum(aux2 * a[..., 1], axis=1)
            J[i0:i0 + BLOCK, 1, 0] -= np.sum(aux2 * a[..., 2], axis=1)
            J[i0:i0 + BLOCK, 1, 2] += np.sum(aux2 * a[..., 0], axis=1)
            J[i0:i0 + BLOCK, 2, 0] += np.sum(aux2 * a[..., 1], axis=1)
            J[i0:i0 + BLOCK, 2, 1] -= np.sum(aux2 * a[..., 0], axis=1)
    return J


def step_seconds(pos, gam, sig, n_targets, kernel="winckelmans", panels=192):
    """Seconds of the reference's NumPy path for one VPM+panel step with free
    wake and stretching at N = len(pos) particles, timed on the first
    n_targets particles as targets (all particles as sources) and scaled by
    N / n_targets (all-pairs work is linear in the target count): three
    velocity sweeps, three Jacobian sweeps (particles.py:122, :148) and the
    velocity sweep at the collocation points and bound-leg centres."""
    n = pos.shape[0]
    t = pos[:n_targets]
    t0 = time.perf_counter()
    velocity_from_particles(t, pos, gam, sig, kernel)
    t_vel = time.perf_counter() - t0
    t0 = time.perf_counter()
    jacobian_from_particles(t, pos, gam, sig, kernel)
    t_jac = time.perf_counter() - t0
    scale = n / n_targets
    step = 3.0 * (t_vel + t_jac) * scale + t_vel * 2 * panels / n_targets
    return step, {"velocity_s": t_vel, "jacobian_s": t_jac, "targets": n_targets, "sources": n}
