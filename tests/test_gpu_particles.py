"""GPU parity of the particle sweeps (kernel.py mirror) against the golden
vectors and the oracle.  FP64: 1e-12 relative (max|d| / max|ref|).  FP32
compensated: 2e-5 relative, the FP32 pair arithmetic's bound on these
inputs (unit round-off 6e-8 times the conditioning of the sums)."""
import numpy as np
import pytest

from fluxvortex_gb300 import _capi
from fluxvortex_gb300 import kernel as K
from oracle import oracle as O
from tests.conftest import rel_err

pytestmark = pytest.mark.gpu
TOL64 = 1e-12
TOL32 = 2e-5


@pytest.mark.parametrize("kernel", ["winckelmans", "gaussianerf"])
def test_golden_velocity(cuda, golden, kernel):
    z = golden("particles_kernel.npz")
    u = K.velocity_from_particles(z["tgt_pos"], z["src_pos"], z["src_gamma"], z["src_sigma"],
                                  kernel)
    assert rel_err(u, z[f"velocity_{kernel}"]) < TOL64


@pytest.mark.parametrize("kernel", ["winckelmans", "gaussianerf"])
def test_golden_jacobian(cuda, golden, kernel):
    z = golden("particles_kernel.npz")
    J = K.jacobian_from_particles(z["tgt_pos"], z["tgt_gamma"], z["src_pos"], z["src_gamma"],
                                  z["src_sigma"], kernel)
    G = z[f"jacobian_{kernel}"]
    assert rel_err(J[150:], G[150:]) < TOL64          # well-conditioned rows
    if kernel == "winckelmans":
        assert rel_err(J, G) < TOL64
    Jo = O.jacobian_from_particles(z["tgt_pos"], z["tgt_gamma"], z["src_pos"], z["src_gamma"],
                                   z["src_sigma"], kernel)
    assert rel_err(J, Jo) < TOL64                      # incl. self pairs


def _field(rng, n, spread=1.0):
    pos = rng.uniform([0, -1, -0.2], [2, 1, 0.2], size=(n, 3)) * spread
    gam = rng.normal(0, 1e-3, size=(n, 3))
    sig = rng.uniform(0.02, 0.08, size=n)
    return pos, gam, sig


MODES = ["velocity", "stretch", "velocity_stretch", "jacobian", "vorticity"]


def _oracle_mode(mode, t, tg, p, g, s, kernel):
    if mode == "velocity":
        return O.velocity_from_particles(t, p, g, s, kernel), None
    if mode == "jacobian":
        return O.jacobian_from_particles(t, tg, p, g, s, kernel).reshape(-1, 9), None
    J = O.jacobian_from_particles(t, tg, p, g, s, kernel)
    if mode == "vorticity":
        w = np.stack([J[:, 2, 1] - J[:, 1, 2], J[:, 0, 2] - J[:, 2, 0], J[:, 1, 0] - J[:, 0, 1]], 1)
        return w, None
    S = np.einsum("tij,tj->ti", J, tg)
    if mode == "stretch":
        return S, None
    return O.velocity_from_particles(t, p, g, s, kernel), S


@pytest.mark.parametrize("precision", ["f64", "f32c"])
@pytest.mark.parametrize("kernel", ["winckelmans", "gaussianerf"])
@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("M,N", [(1, 1), (257, 513), (4096, 3001)])
def test_modes_vs_oracle(cuda, precision, kernel, mode, M, N):
    rng = np.random.default_rng(M * 31 + N)
    p, g, s = _field(rng, N)
    t = np.vstack([p[: M // 2], rng.uniform([0, -1, -0.2], [2, 1, 0.2], size=(M - M // 2, 3))])
    tg = rng.normal(0, 1e-3, size=(M, 3))
    mid = getattr(_capi, "PAIR_" + mode.upper())
    a, b = K.particle_pairs(mid, t, tg, p, g, s, kernel, precision)
    oa, ob = _oracle_mode(mode, t, tg, p, g, s, kernel)
    tol = TOL64 if precision == "f64" else TOL32
    assert rel_err(a, oa) < tol
    if ob is not None:
        assert rel_err(b, ob) < tol


def test_torch_path_and_empty(cuda):
    import torch
    rng = np.random.default_rng(3)
    p, g, s = _field(rng, 1000)
    t = rng.uniform(0, 1, size=(300, 3))
    ut = K.velocity_from_particles(torch.as_tensor(t, device=cuda), torch.as_tensor(p, device=cuda),
                                   torch.as_tensor(g, device=cuda), torch.as_tensor(s, device=cuda),
                                   "winckelmans")
    assert ut.is_cuda
    uo = O.velocity_from_particles(t, p, g, s, "winckelmans")
    assert rel_err(ut.cpu().numpy(), uo) < TOL64
    u0 = K.velocity_from_particles(t, np.zeros((0, 3)), np.zeros((0, 3)), np.zeros(0))
    assert u0.shape == (300, 3) and not u0.any()


def test_f32c_far_from_origin(cuda):
    """Re-centring keeps FP32 accurate for a compact cluster far from the
    origin (slab coordinates up to 20 chords)."""
    rng = np.random.default_rng(9)
    p, g, s = _field(rng, 2048)
    p = p * 0.2 + np.array([18.0, 7.0, 1.0])
    u32 = K.velocity_from_particles(p, p, g, s, "winckelmans", "f32c")
    u64 = K.velocity_from_particles(p, p, g, s, "winckelmans", "f64")
    assert rel_err(u32, u64) < TOL32
