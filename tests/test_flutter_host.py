"""Host side of the flutter sweep (CPU): beam model against the beam oracle,
envelope growth and flutter-speed interpolation, span interpolation weights."""
import numpy as np

from fluxvortex_gb300.beam import BeamModel
from fluxvortex_gb300.flutter import (envelope_growth, flutter_speed, goland, interp_weights)
from oracle.beam import Beam, distribute


def test_beam_model_matches_oracle():
    cfg = goland()
    m = cfg.beam_model()
    o = Beam(**cfg.beam)
    f = o.free
    np.testing.assert_allclose(m.Kr, o.K[np.ix_(f, f)], rtol=1e-13, atol=1e-13 * np.abs(o.K).max())
    np.testing.assert_allclose(m.Mr, o.M[np.ix_(f, f)], rtol=1e-13, atol=1e-13 * np.abs(o.M).max())
    np.testing.assert_allclose(m.Cr, o.C[np.ix_(f, f)], rtol=1e-9, atol=1e-12 * np.abs(o.C).max())
    np.testing.assert_allclose(m.frequencies(), o.frequencies(), rtol=1e-9)
    # Newmark through the precomputed inverse == the oracle's dense solve
    dt = cfg.dt
    Kinv = m.newmark_inverse(dt)
    d, v, a = m.initial_state(0.05, np.radians(2.0))
    o.d[:], o.v[:], o.a[:] = d, v, a
    F = np.zeros(m.ndof)
    F[3::3] = 1200.0
    F[5::3] = -80.0
    b, g = 0.25, 0.5
    for _ in range(20):
        dr, vr, ar = d[f], v[f], a[f]
        feff = (F[f] + m.Mr @ (dr / (b * dt * dt) + vr / (b * dt) + (1 / (2 * b) - 1) * ar)
                + m.Cr @ (g / (b * dt) * dr + (g / b - 1) * vr + dt * (g / (2 * b) - 1) * ar))
        dn = Kinv @ feff
        an = (dn - dr) / (b * dt * dt) - vr / (b * dt) - (1 / (2 * b) - 1) * ar
        vn = vr + dt * ((1 - g) * ar + g * an)
        d[f], v[f], a[f] = dn, vn, an
        o.step(F, dt)
    assert np.abs(d - o.d).max() <= 1e-10 * np.abs(o.d).max()
    assert np.abs(v - o.v).max() <= 1e-9 * np.abs(o.v).max()


def test_envelope_growth_recovers_rate():
    dt = 0.003
    t = np.arange(800) * dt
    for rate in (-1.5, -0.2, 0.3, 2.0):
        sig = np.exp(rate * t) * np.sin(2 * np.pi * 7.7 * t + 0.3)
        assert abs(envelope_growth(sig, dt) - rate) < 0.02 * max(1.0, abs(rate))
    assert envelope_growth(np.ones(5), dt) == 0.0


def test_flutter_speed_interpolation():
    V = np.array([80.0, 100.0, 120.0, 140.0])
    s = np.array([-2.0, -1.0, 1.0, 3.0])
    assert abs(flutter_speed(V, s) - 110.0) < 1e-12
    assert flutter_speed(V, -np.abs(s)) is None
    # unsorted input
    assert abs(flutter_speed(V[::-1], s[::-1]) - 110.0) < 1e-12


def test_interp_weights_match_numpy_and_distribute():
    y = np.linspace(0.0, 6.096, 9)
    q = np.array([0.0, 0.3, 0.762, 3.0, 6.0, 6.096])
    k, xi = interp_weights(q, y)
    f = np.sin(y) + 2.0
    np.testing.assert_allclose(f[k] * (1 - xi) + f[k + 1] * xi, np.interp(q, y, f), rtol=1e-14)
    lift = np.arange(1.0, 7.0)
    F = distribute(y, q, lift, 0.5 * lift)
    G = np.zeros(27)
    for j in range(len(q)):
        G[3 * k[j]] += lift[j] * (1 - xi[j])
        G[3 * (k[j] + 1)] += lift[j] * xi[j]
        G[3 * k[j] + 2] += 0.5 * lift[j] * (1 - xi[j])
        G[3 * (k[j] + 1) + 2] += 0.5 * lift[j] * xi[j]
    np.testing.assert_allclose(F, G, rtol=1e-14)
