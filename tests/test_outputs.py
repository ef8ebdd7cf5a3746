"""Output files in the reference's layouts (fluxvortex_gb300.outputs)."""
import types

import numpy as np

from fluxvortex_gb300 import outputs as OUT


def test_force_history_layout_and_merge(tmp_path, golden):
    path = str(tmp_path / "flapping_results.npz")
    ref = golden("flapping_history.npz")
    # a run given as (t, cl, cdi) and one as a step-like object
    OUT.save_force_history(path, {"ps": (ref["t_ps"], ref["cl_ps"], ref["cdi_ps"])})
    run = types.SimpleNamespace(cl=ref["cl_h10"], cdi=ref["cdi_h10"],
                                cfg=types.SimpleNamespace(dt=1.0 / 43))
    OUT.save_force_history(path, {"h10": run})
    z = np.load(path, allow_pickle=False)
    assert set(z.files) == {"t_ps", "cl_ps", "cdi_ps", "t_h10", "cl_h10", "cdi_h10"}
    assert np.array_equal(z["cl_ps"], ref["cl_ps"]) and np.array_equal(z["cl_h10"], ref["cl_h10"])
    assert np.allclose(z["t_h10"], ref["t_h10"], rtol=0, atol=1e-12)
    back = OUT.load_force_history(path)
    assert sorted(back) == ["h10", "ps"]


def test_force_coefficients_sign_convention():
    c = OUT.force_coefficients_W([0.5, 0.6], [0.01, 0.02])
    assert c.shape == (2, 3)
    assert np.array_equal(-c[:, 2], [0.5, 0.6])      # CL = -c[2]
    assert np.array_equal(-c[:, 0], [0.01, 0.02])    # CDi = -c[0]


def test_flutter_tips_and_particle_snapshot(tmp_path):
    sweep = types.SimpleNamespace(
        V=np.array([100.0, 160.0]), cfg=types.SimpleNamespace(dt=0.003),
        histories=lambda: ([np.arange(5.0), np.arange(7.0)], [np.zeros(5), np.ones(7)]),
        sigma=lambda: np.array([-0.1, 0.2]), flutter_speed=lambda: 140.2)
    OUT.save_flutter_tips(str(tmp_path / "tips.npz"), sweep)
    z = np.load(tmp_path / "tips.npz", allow_pickle=False)
    assert z["w_tip_160.0"].shape == (7,) and np.array_equal(z["theta_tip_100.0"], np.zeros(5))
    assert float(z["flutter_speed"]) == 140.2 and float(z["dt"]) == 0.003
    field = types.SimpleNamespace(positions=np.ones((3, 3)), gammas=np.zeros((3, 3)),
                                  sigmas=np.full(3, 0.1), ages=np.arange(3.0), np=3)
    OUT.save_particles(str(tmp_path / "p.npz"), field, t=0.5)
    p = np.load(tmp_path / "p.npz", allow_pickle=False)
    assert int(p["np"]) == 3 and float(p["t"]) == 0.5 and p["pos"].shape == (3, 3)


def test_flutter_data_layout_round_trip(tmp_path):
    """save_flutter_data writes the reference's figures/flutter_data.npz
    layout (tests/animate_flutter.py:161-168): per-node (steps x nodes) heave
    and twist at a stable and a fluttering airspeed, y_nodes, dt.  The
    reference's file (60 chords at 100 and 160 m/s, its coupling records
    n_steps - 2 steps) holds (364, 9) and (227, 9) arrays."""
    from fluxvortex_gb300.flutter import goland
    cfg = goland(num_chords=60.0, coupling="reference")
    steps = {100.0: cfg.n_steps(100.0) - 2, 160.0: cfg.n_steps(160.0) - 2}
    assert steps == {100.0: 364, 160.0: 227}
    y = np.linspace(0.0, 6.096, 9)
    hist = {e: (np.random.default_rng(e).standard_normal((n, 9)),
                np.random.default_rng(10 + e).standard_normal((n, 9)))
            for e, n in enumerate(steps.values())}
    sweep = types.SimpleNamespace(V=np.array([100.0, 160.0]), cfg=cfg,
                                  beam=types.SimpleNamespace(y_nodes=y),
                                  node_histories=lambda e: hist[e])
    OUT.save_flutter_data(str(tmp_path / "flutter_data.npz"), sweep, 100.0, 160.0)
    z = np.load(tmp_path / "flutter_data.npz", allow_pickle=False)
    assert sorted(z.files) == sorted(["w_stable", "theta_stable", "w_flutter", "theta_flutter",
                                      "y_nodes", "dt"])
    assert z["w_stable"].shape == z["theta_stable"].shape == (364, 9)
    assert z["w_flutter"].shape == z["theta_flutter"].shape == (227, 9)
    assert z["y_nodes"].shape == (9,) and float(z["dt"]) == 0.003
    d = OUT.load_flutter_data(str(tmp_path / "flutter_data.npz"))
    assert np.array_equal(d["stable"]["w_history"], hist[0][0])
    assert np.array_equal(d["flutter"]["theta_history"], hist[1][1])
    assert np.array_equal(d["flutter"]["y_nodes"], y) and d["stable"]["dt"] == 0.003
