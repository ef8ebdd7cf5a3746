"""Seeded synthetic workloads with the shapes of the reference's benchmark cases.

``slab_wake(n)``: the synthetic Biot-Savart sweep -- n vortex particles
uniform in a 20c x 10c x 2c slab behind a unit-chord wing (x in [1, 21],
y in [-5, 5], z in [-1, 1]), vector strengths i.i.d. N(0, (1e-3 m^3/s)^2)
per component, core radius 0.02c, plus 4096 collocation targets on a planar
64 x 64 grid over the wing (x in [0, 1], y in [-5, 5], z = 0).  The
reference measures nothing at this scale; these inputs stand in for its wake
runs with its stated shapes and value distributions.  ``x0`` moves the slab's
upstream face (default: one chord behind the leading edge), e.g. behind the
ring rows of a larger configuration.

``resolved_core(n)``: 1.3 x the slab's mean particle spacing, the core with
which a seeded slab stands in for a grown wake (converted particles take 1.3
x their ring's mean edge): cores that overlap their neighbours keep the
stretching term bounded, while the 0.02c cores of the sweep case sit below
the spacing (0.074c at 2^20) and their stretching blows up within a cycle.

``AIRCRAFT_SLAB_X0``: the slab's upstream face behind the large flapping
configuration -- past the V-tail's trailing edge (x = 6.5) and its N_keep = 10
ring rows (10 dt V = 2.3 m), so that the seeded particles fill the far wake
and not the surfaces.
"""
from __future__ import annotations

import numpy as np

SEED = 20261203
AIRCRAFT_SLAB_X0 = 9.0


def resolved_core(n: int, chord: float = 1.0) -> float:
    return 1.3 * (20.0 * 10.0 * 2.0 / max(n, 1)) ** (1.0 / 3.0) * chord


def slab_wake(n: int, seed: int = SEED, chord: float = 1.0, x0: float = 1.0, sigma=None):
    rng = np.random.default_rng(seed)
    lo = np.array([x0, -5.0, -1.0]) * chord
    hi = np.array([x0 + 20.0, 5.0, 1.0]) * chord
    pos = rng.uniform(lo, hi, size=(n, 3))
    gamma = rng.normal(0.0, 1e-3, size=(n, 3))
    sigma = np.full(n, 0.02 * chord if sigma is None else float(sigma))
    g = (np.arange(64) + 0.5) / 64.0
    xs = g * chord
    ys = -5.0 * chord + g * 10.0 * chord
    X, Y = np.meshgrid(xs, ys, indexing="ij")
    colloc = np.stack([X.ravel(), Y.ravel(), np.zeros(X.size)], axis=1)
    return pos, gamma, sigma, colloc
