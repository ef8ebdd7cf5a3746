"""The PteraSoftware-free geometry of the large flapping configuration
(three lifting surfaces in one grid) and the oracle's step on it against the
reference's own recorded CL / CDi histories (tests/golden/flapping_history.npz,
from the reference's figures/flapping_results.npz).  The histories come from
PteraSoftware's panels, so the check is qualitative: correlation, last-cycle
mean and amplitude."""
import numpy as np
import pytest

from fluxvortex_gb300.geometry import (Kinematics, combine, flapping_aircraft, heaving_wing,
                                       lattice, rectangular_wing)


def test_layout_of_three_surfaces():
    cfg = flapping_aircraft()
    col, surf, kins = cfg.layout()
    assert cfg.verts.shape == (7, 35, 3)
    assert col.size == 32 and len(kins) == 3
    assert np.array_equal(np.bincount(surf), [9, 9, 17])
    # no strip spans two surfaces
    assert np.all(surf[col] == surf[col + 1])
    L = lattice(cfg.vertices(0.0), col)
    assert L.colloc.shape == (192, 3) and L.te_back.shape == (35, 3)
    assert np.all(L.normal[:, 2] > 0.85)
    # the main halves are mirror images with a 1 m gap at the root
    left, right = cfg.verts[:, :9], cfg.verts[:, 9:18]
    assert np.allclose(left[:, ::-1, 1], -right[:, :, 1])
    assert np.isclose(right[0, 0, 1], 0.5) and np.isclose(left[0, -1, 1], -0.5)
    assert np.isclose(cfg.s_ref, 0.5 * (1.75 + 1.5) * 6.0, rtol=2e-2)


def test_one_surface_layout_is_the_plain_grid():
    cfg = heaving_wing()
    col, surf, kins = cfg.layout()
    assert np.array_equal(col, np.arange(cfg.verts.shape[1] - 1))
    verts, col2, surf2 = combine([cfg.verts])
    assert np.array_equal(col, col2) and np.array_equal(surf, surf2)
    a, b = lattice(cfg.verts), lattice(cfg.verts, col)
    for f in ("br", "fr", "fl", "bl", "colloc", "normal", "area", "te_back"):
        assert np.array_equal(getattr(a, f), getattr(b, f))


@pytest.mark.parametrize("flapping", ["right", "both"])
def test_body_velocity_is_the_time_derivative_of_the_panels(flapping):
    cfg = flapping_aircraft(flapping=flapping)
    col = cfg.layout()[0]
    t, e = 0.137, 1e-6
    fd = (lattice(cfg.vertices(t + e), col).colloc
          - lattice(cfg.vertices(t - e), col).colloc) / (2 * e)
    v = cfg.point_velocity(lattice(cfg.vertices(t), col).colloc, t)
    assert np.abs(fd - v).max() < 1e-7 * np.abs(v).max()
    moving = np.abs(v).max(axis=1) > 0
    n_moving = {"right": 48, "both": 96}[flapping]
    assert moving.sum() == n_moving


def test_hinge_offset_flapping_keeps_the_root_on_its_hinge():
    k = Kinematics(flap_amp=np.radians(15.0), period=1.0, y0=0.5)
    half = rectangular_wing(1.0, 3.0, 2, 3, symmetric=False, y0=0.5)
    v = k.vertices(half, 0.25)                      # theta = 15 deg
    assert np.allclose(v[:, 0, 1:], half[:, 0, 1:])  # root column on the hinge line
    tip = v[0, -1]
    assert np.isclose(tip[1], 0.5 + 3.0 * np.cos(np.radians(15.0)))
    assert np.isclose(tip[2], 3.0 * np.sin(np.radians(15.0)))
    mirror = half.copy()
    mirror[..., 1] *= -1
    vm = k.vertices(mirror, 0.25)
    assert np.allclose(vm[..., 1], -v[..., 1]) and np.allclose(vm[..., 2], v[..., 2])


def test_oracle_tracks_the_reference_flapping_history(golden):
    """129 steps of the FP64 oracle, prescribed particle wake (the recorded
    hybrid run's form), against the reference's N_keep = 10 history.  The
    reference's step 0 is a wake-free start, so its step k + 1 is this step
    k; the first three steps (the start transient) are left out."""
    from oracle.hybrid import HybridOracle
    ref = golden("flapping_history.npz")
    cfg = flapping_aircraft(free_vpm=False)
    o = HybridOracle(cfg)
    for _ in range(129):
        o.step()
    cl, cdi = np.array(o.cl)[3:-1], np.array(o.cdi)[3:-1]
    rcl, rcdi = ref["cl_h10"][4:], ref["cdi_h10"][4:]
    assert np.corrcoef(cl, rcl)[0, 1] > 0.998
    assert np.corrcoef(cdi, rcdi)[0, 1] > 0.98
    last, rlast = cl[-43:], rcl[-43:]
    assert abs(last.mean() / rlast.mean() - 1.0) < 0.02
    amp = lambda x: 0.5 * (x.max() - x.min())  # noqa: E731
    assert abs(amp(last) / amp(rlast) - 1.0) < 0.08
    assert abs(cdi[-43:].mean() / rcdi[-43:].mean() - 1.0) < 0.1


def test_bernoulli_lift_matches_kutta_joukowski_on_the_static_wing():
    """The two load paths of the oracle integrate the same circulation: the
    lift agrees (the drag differs: normal pressure carries no suction)."""
    from fluxvortex_gb300.geometry import static_wing
    from oracle.hybrid import HybridOracle
    cl = {}
    for loads in ("kj", "bernoulli"):
        o = HybridOracle(static_wing(free_vpm=False, loads=loads))
        for _ in range(12):
            o.step()
        cl[loads] = np.array(o.cl)
    assert np.abs(cl["bernoulli"][3:] / cl["kj"][3:] - 1.0).max() < 2e-3
