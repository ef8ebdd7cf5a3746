"""Seeded synthetic workloads with the shapes of the reference's benchmark cases.

``slab_wake(n)``: the synthetic Biot-Savart sweep -- n vortex particles
uniform in a 20c x 10c x 2c slab behind a unit-chord wing (x in [1, 21],
y in [-5, 5], z in [-1, 1]), vector strengths i.i.d. N(0, (1e-3 m^3/s)^2)
per component, core radius 0.02c, plus 4096 collocation targets on a planar
64 x 64 grid over the wing (x in [0, 1], y in [-5, 5], z = 0).  The
reference measures nothing at this scale; these inputs stand in for its wake
runs with its stated shapes and value distributions.
"""
from __future__ import annotations

import numpy as np

SEED = 20261203


def slab_wake(n: int, seed: int = SEED, chord: float = 1.0):
    rng = np.random.default_rng(seed)
    lo = np.array([1.0, -5.0, -1.0]) * chord
    hi = np.array([21.0, 5.0, 1.0]) * chord
    pos = rng.uniform(lo, hi, size=(n, 3))
    gamma = rng.normal(0.0, 1e-3, size=(n, 3))
    sigma = np.full(n, 0.02 * chord)
    g = (np.arange(64) + 0.5) / 64.0
    xs = g * chord
    ys = -5.0 * chord + g * 10.0 * chord
    X, Y = np.meshgrid(xs, ys, indexing="ij")
    colloc = np.stack([X.ravel(), Y.ravel(), np.zeros(X.size)], axis=1)
    return pos, gamma, sigma, colloc
