"""Device VortexParticleField against the oracle's restatement of
particles.py:85-246 (RK3 + rVPM + clamps + NaN guard + relaxation) and
against the reference's own outputs where the reference is well conditioned.
FP64 integration; tolerance 1e-11 relative after two steps (the relaxation's
normalisation amplifies 1e-13 sweep differences by up to ~10x)."""
import numpy as np
import pytest

from fluxvortex_gb300.particles import VortexParticleField
from oracle import oracle as O
from tests.conftest import rel_err

pytestmark = pytest.mark.gpu

CASES = [(k, s, f, r) for k in ("winckelmans", "gaussianerf")
         for s, f, r in ((1, 1, 1), (0, 1, 1), (0, 0, 1), (1, 1, 0), (0, 1, 0))]


def _run_gpu(z, kernel, s, f, r, precision="f64", steps=2):
    n = len(z["sigma0"])
    fld = VortexParticleField(max_particles=n + 7, nu=1e-4 if s else 0.0,
                              rlxf=0.3 if r else 0.0, kernel=kernel, precision=precision)
    fld.add_particles_batch(z["pos0"], z["gamma0"], z["sigma0"])
    for _ in range(steps):
        fld.advect_rk3(float(z["dt"]), z["u_inf"], stretch=bool(s), free_wake=bool(f))
    return fld


@pytest.mark.parametrize("kernel,s,f,r", CASES)
def test_rk3_vs_oracle(cuda, golden, kernel, s, f, r):
    z = golden("particles_rk3.npz")
    fld = _run_gpu(z, kernel, s, f, r)
    p, g, sg, a = z["pos0"], z["gamma0"], z["sigma0"], np.zeros(len(z["sigma0"]))
    for _ in range(2):
        p, g, sg, a = O.advect_rk3(p, g, sg, a, float(z["dt"]), z["u_inf"], kernel,
                                   1e-4 if s else 0.0, 0.3 if r else 0.0, bool(s), bool(f))
    assert rel_err(fld.positions, p) < 1e-13
    assert rel_err(fld.gammas, g) < 1e-11
    assert rel_err(fld.sigmas, sg) < 1e-12
    assert np.allclose(fld.ages, a, rtol=0, atol=1e-15)


@pytest.mark.parametrize("kernel,s,f,r", [c for c in CASES
                                          if c[3] == 0 and (c[0] == "winckelmans" or c[1] == 0)])
def test_rk3_vs_reference_golden(cuda, golden, kernel, s, f, r):
    """Cases where the reference itself is well conditioned: its own numbers."""
    z = golden("particles_rk3.npz")
    fld = _run_gpu(z, kernel, s, f, r)
    tag = f"{kernel}_s{s}_f{f}_r{r}"
    assert rel_err(fld.positions, z["pos_" + tag]) < 1e-13
    assert rel_err(fld.gammas, z["gamma_" + tag]) < 1e-11
    assert rel_err(fld.sigmas, z["sigma_" + tag]) < 1e-12


def test_rk3_f32c_close_to_f64(cuda, golden):
    z = golden("particles_rk3.npz")
    a = _run_gpu(z, "winckelmans", 1, 1, 1, "f64")
    b = _run_gpu(z, "winckelmans", 1, 1, 1, "f32c")
    assert rel_err(b.positions, a.positions) < 1e-7
    assert rel_err(b.gammas, a.gammas) < 1e-4


def test_capacity_and_nan_guard(cuda):
    from fluxvortex_gb300 import _capi
    fld = VortexParticleField(max_particles=4, kernel="winckelmans")
    fld.add_particles_batch(np.zeros((3, 3)) + [[0, 0, 0], [1, 0, 0], [0, 1, 0]],
                            np.ones((3, 3)) * 1e-2, np.full(3, 0.1))
    with pytest.raises(RuntimeError):
        fld.add_particles_batch(np.zeros((2, 3)), np.zeros((2, 3)), np.ones(2))
    fld.add_particle([0, 0, 1.0], [np.inf, 0, 0], 0.1)   # a non-finite strength
    _capi.status_read_and_clear()
    fld.advect_rk3(0.01, [1.0, 0, 0], stretch=False, free_wake=False)
    g = fld.gammas
    assert np.all(g[3] == 0.0) and np.all(np.isfinite(g))
    assert _capi.status_read_and_clear() & 2


def test_velocity_clamp(cuda):
    fld = VortexParticleField(max_particles=2, kernel="winckelmans", rlxf=0.0)
    fld.add_particle([0, 0, 0], [0, 0, 0], 0.1)
    fld.advect_rk3(0.01, [100.0, 0, 0], stretch=False, free_wake=False)
    # |U| clamped to 50: x advances by 50 * dt over the step
    assert abs(fld.positions[0, 0] - 0.5) < 1e-12
