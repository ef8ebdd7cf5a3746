"""Particle population control on the device (fvx_vpm_drop_oldest,
fvx_vpm_merge_pass) against the reference's own merge pass
(tests/golden/population_merge.npz, from newton_pc/adapters/flap.py:478-563)
and the oracle; the hybrid step with population control against the hybrid
oracle."""
import numpy as np
import pytest
import torch

from fluxvortex_gb300.geometry import heaving_wing
from fluxvortex_gb300.hybrid import HybridStep
from fluxvortex_gb300.particles import VortexParticleField
from oracle import population as POP
from oracle.hybrid import HybridOracle

pytestmark = pytest.mark.gpu


def _field(pos, alpha, sigma, age=None):
    f = VortexParticleField(pos.shape[0] + 16, kernel="winckelmans", device="cuda")
    f.add_particles_batch(pos, alpha, sigma)
    if age is not None:
        f._age[: pos.shape[0]].copy_(torch.as_tensor(age))
    return f


@pytest.mark.parametrize("case", ["count", "dist", "tight"])
def test_merge_pass_matches_reference(cuda, golden, case):
    z = golden("population_merge.npz")
    n = z["sigma"].shape[0]
    f = _field(z["pos"], z["alpha"], z["sigma"], np.arange(n, dtype=float))
    m = f.merge_pass(z["ref"], float(z["speed"]), float(z[case + "_eps"]),
                     int(z[case + "_protect"]), float(z[case + "_dist"]) or None)
    assert m == int(z[case + "_merged"])
    assert f.np == n - m
    assert np.array_equal(f.positions, z[case + "_pos"])
    assert np.array_equal(f.gammas, z[case + "_alpha"])
    assert np.array_equal(f.sigmas, z[case + "_sigma"])
    # ages follow the survivors (the first particle of each merged pair)
    _, _, _, age, _ = POP.merge_pass(z["pos"], z["alpha"], z["sigma"], np.arange(n, dtype=float),
                                     z["ref"], float(z["speed"]), float(z[case + "_eps"]),
                                     int(z[case + "_protect"]), float(z[case + "_dist"]) or None)
    assert np.array_equal(f.ages, age)


def test_merge_pass_gates_and_drop(cuda):
    rng = np.random.default_rng(5)
    n = 100
    pos = rng.uniform(1.0, 2.0, (n, 3))
    alpha = np.tile([0.0, 1e-3, 0.0], (n, 1))
    sigma = np.full(n, 0.1)
    ref = np.array([[0.5, 0.0, 0.0]])
    f = _field(pos, alpha, sigma)
    assert f.merge_pass(ref, 10.0, 1e-3, protect_newest=60) == 0      # n < 2 protect
    assert f.np == n
    assert f.merge_pass(ref, 10.0, 1e-3, protect_dist=50.0) == 0      # < 4 candidates
    dropped = f.drop_oldest(30)
    assert dropped == 70 and f.np == 30
    assert np.array_equal(f.positions, pos[70:])
    assert f.drop_oldest(40) == 0


def test_hybrid_step_with_drop_matches_oracle(cuda):
    cfg = heaving_wing(n_keep=3, free_vpm=True, population="drop", pop_max=150)
    g, o = HybridStep(cfg, precision="f64"), HybridOracle(cfg)
    for _ in range(10):
        g.step()
        o.step()
    assert g.field.np == o.p_pos.shape[0] == 150
    assert np.abs(np.array(g.cl) - np.array(o.cl)).max() < 1e-10 * np.abs(o.cl).max()
    assert np.abs(g.field.positions - o.p_pos).max() < 1e-10


def test_hybrid_step_with_merge_conserves_strength(cuda):
    """Prescribed particle wake: merging changes the count but conserves the
    total strength, and the loads stay close to the run without merging."""
    kw = dict(n_keep=3, free_vpm=False, stretch=False)
    plain = HybridStep(heaving_wing(**kw), precision="f64")
    merged = HybridStep(heaving_wing(population="merge", merge_eps=1e-2, merge_protect=8, **kw),
                        precision="f64")
    for _ in range(14):
        plain.step()
        merged.step()
    assert merged.n_merged > 0
    assert merged.field.np == plain.field.np - merged.n_merged
    a, b = plain.field.gammas.sum(0), merged.field.gammas.sum(0)
    assert np.abs(a - b).max() < 1e-12 * np.abs(plain.field.gammas).sum()
    assert np.abs(np.array(merged.cl) - np.array(plain.cl)).max() < 1e-2 * np.abs(plain.cl).max()
