"""Device hybrid panel-particle step against the oracle's restatement of the
reference's HybridSolver step (oracle/hybrid.py).  FP64: CL / CDi histories
within 1e-10 of the largest |CL| (the spec bar on the CL/CDi time
history); strengths and particle states within 1e-10 relative.  FP32
compensated particle sweeps: CL within 1e-4."""
import numpy as np
import pytest

from fluxvortex_gb300.geometry import flapping_aircraft, heaving_wing, static_wing
from fluxvortex_gb300.hybrid import HybridStep
from oracle.hybrid import HybridOracle
from tests.conftest import rel_err

pytestmark = pytest.mark.gpu


def _run(cfg, steps, precision="f64"):
    g = HybridStep(cfg, precision=precision)
    o = HybridOracle(cfg)
    for _ in range(steps):
        g.step()
        o.step()
    return g, o


def _hist_err(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / np.max(np.abs(b)))


@pytest.mark.parametrize("stretch,free,rlxf,rule", [(False, True, 0.0, "v_dt"),
                                                    (True, True, 0.0, "edge"),
                                                    (False, False, 0.3, "v_dt")])
def test_heaving_wing_fp64(cuda, stretch, free, rlxf, rule):
    cfg = heaving_wing(n_keep=4, free_vpm=free, stretch=stretch, rlxf=rlxf, sigma_rule=rule)
    g, o = _run(cfg, 16)
    assert g.field.np == o.p_pos.shape[0] > 0
    assert _hist_err(g.cl, o.cl) < 1e-10
    assert _hist_err(g.cdi, o.cdi) < 1e-10
    assert rel_err(g.gamma.cpu().numpy(), o.gamma) < 1e-10
    assert rel_err(g.field.positions, o.p_pos) < 1e-10
    assert rel_err(g.field.gammas, o.p_gam) < 1e-10
    assert rel_err(g.field.sigmas, o.p_sig) < 1e-10


def test_static_wing_fp64(cuda):
    cfg = static_wing(free_vpm=False)
    g, o = _run(cfg, 12)
    assert _hist_err(g.cl, o.cl) < 1e-10
    assert _hist_err(g.cdi, o.cdi) < 1e-10
    assert 0.3 < g.cl[-1] < 0.5


def test_heaving_wing_f32c_cl_within_1e4(cuda):
    cfg = heaving_wing(n_keep=4, free_vpm=True)
    g64 = HybridStep(cfg, precision="f64")
    g32 = HybridStep(cfg, precision="f32c")
    for _ in range(20):
        g64.step()
        g32.step()
    assert _hist_err(g32.cl, g64.cl) < 1e-4
    assert _hist_err(g32.cdi, g64.cdi) < 1e-3


@pytest.mark.parametrize("flapping,free,stretch,steps", [("right", False, False, 12),
                                                         ("both", True, False, 12),
                                                         ("both", True, True, 8)])
def test_flapping_aircraft_fp64(cuda, flapping, free, stretch, steps):
    """Three surfaces (two main-wing halves with a gap between their roots, a
    V-tail of 16 strips) in one grid: per-surface kinematics, per-surface
    trailing edges and wake strips, conversion with the strip map.  With free
    wake and stretching the converted particles (|alpha| up to ~80, sigma
    ~0.2) amplify round-off by 10-30x per step once they act on each other
    (1e-15 at step 5, 1e-8 at step 11), so that case stops at step 8."""
    cfg = flapping_aircraft(n_keep=4, flapping=flapping, free_vpm=free, stretch=stretch)
    g, o = _run(cfg, steps)
    assert g.P == 192
    assert g.field.np == o.p_pos.shape[0] == (steps - 4) * 32 * 4
    assert _hist_err(g.cl, o.cl) < 1e-10
    assert _hist_err(g.cdi, o.cdi) < 1e-10
    assert rel_err(g.gamma.cpu().numpy(), o.gamma) < 1e-10
    assert rel_err(g.field.positions, o.p_pos) < 1e-10
    assert rel_err(g.field.gammas, o.p_gam) < 1e-10


def test_snapshot_restore_resumes_bitwise(cuda, tmp_path):
    """A device snapshot, and a host snapshot written with numpy.savez and read
    back, both resume the step bitwise (FP64 direct sweeps and the panel side
    reduce in a fixed order)."""
    cfg = flapping_aircraft(n_keep=3, flapping="both", free_vpm=True, stretch=True)
    g = HybridStep(cfg, precision="f64")
    for _ in range(5):
        g.step()
    dev = g.snapshot()
    host = g.snapshot(host=True)
    flat = {k: v for k, v in host.items() if k != "field"}
    flat.update({"field_" + k: v for k, v in host["field"].items()})
    np.savez(tmp_path / "state.npz", **flat)
    for _ in range(4):
        g.step()
    ref = (g.cl.copy(), g.cdi.copy(), g.field.positions, g.field.gammas, g.field.sigmas)
    assert g.field.np > host["field"]["np"] > 0

    def again(state):
        g.restore(state)
        for _ in range(4):
            g.step()
        got = (g.cl, g.cdi, g.field.positions, g.field.gammas, g.field.sigmas)
        for a, b in zip(got, ref):
            assert np.array_equal(a, b)

    again(dev)
    z = np.load(tmp_path / "state.npz")
    st = {k: z[k] for k in z.files if not k.startswith("field_")}
    st["field"] = {k[6:]: z[k] for k in z.files if k.startswith("field_")}
    again(st)


@pytest.mark.parametrize("P,nsys", [(1, 1), (7, 3), (120, 2), (164, 1), (192, 3), (300, 2), (600, 1)])
def test_lu_solve_batched_matches_numpy(cuda, P, nsys):
    """The batched FP64 solve (partial pivoting) against numpy.linalg.solve on
    diagonally weak random systems whose first pivot needs a row swap."""
    import torch
    from fluxvortex_gb300 import _capi
    rng = np.random.default_rng(P)
    A = rng.standard_normal((nsys, P, P)) + 0.5 * np.eye(P)
    if P > 1:
        A[:, 0, 0] = 0.0                           # forces a swap at k = 0
    b = rng.standard_normal((nsys, P))
    x = np.stack([np.linalg.solve(A[i], b[i]) for i in range(nsys)])
    dA = torch.as_tensor(A, device="cuda").contiguous()
    db = torch.as_tensor(b, device="cuda").contiguous()
    _capi.check(_capi.load().fvx_lu_solve_batched(nsys, P, dA.data_ptr(), db.data_ptr(), None))
    got = db.cpu().numpy()
    assert _capi.status_read_and_clear() == 0
    assert np.abs(got - x).max() <= 1e-9 * np.abs(x).max()


@pytest.mark.parametrize("P,nsys", [(1, 1), (7, 3), (120, 2), (192, 3)])
def test_lu_factor_then_solve_is_the_fused_solve_bit_for_bit(cuda, P, nsys):
    """The factorisation on its own (A left unchanged) and the replayed solve
    give the fused solve's solution bit for bit; sizes past 192 are refused."""
    import torch
    from fluxvortex_gb300 import _capi
    lib = _capi.load()
    rng = np.random.default_rng(100 + P)
    A = rng.standard_normal((nsys, P, P)) + 0.5 * np.eye(P)
    if P > 1:
        A[:, 0, 0] = 0.0
    b = rng.standard_normal((nsys, P))
    dA = torch.as_tensor(A, device="cuda").contiguous()
    db = torch.as_tensor(b, device="cuda").contiguous()
    fused_A, fused_b = dA.clone(), db.clone()
    _capi.check(lib.fvx_lu_solve_batched(nsys, P, fused_A.data_ptr(), fused_b.data_ptr(), None))
    wb = int(lib.fvx_lu_workspace_bytes(P))
    assert wb == 8 * (P * P + P + P * (P + 1) // 2)
    work = torch.empty(nsys * wb // 8, dtype=torch.float64, device="cuda")
    A0 = dA.clone()
    _capi.check(lib.fvx_lu_factor_batched(nsys, P, dA.data_ptr(), work.data_ptr(), None))
    _capi.check(lib.fvx_lu_solve_factored_batched(nsys, P, work.data_ptr(), db.data_ptr(), None))
    torch.cuda.synchronize()
    assert _capi.status_read_and_clear() == 0
    assert torch.equal(dA, A0)
    assert torch.equal(db, fused_b)
    assert lib.fvx_lu_workspace_bytes(193) == 0
    with pytest.raises(_capi.FvxError):
        _capi.check(lib.fvx_lu_factor_batched(1, 193, dA.data_ptr(), work.data_ptr(), None))


def test_lu_solve_flags_a_singular_system_and_refuses_oversize(cuda):
    import torch
    from fluxvortex_gb300 import _capi
    lib = _capi.load()
    A = torch.zeros((1, 4, 4), dtype=torch.float64, device="cuda")
    b = torch.ones((1, 4), dtype=torch.float64, device="cuda")
    _capi.check(lib.fvx_lu_solve_batched(1, 4, A.data_ptr(), b.data_ptr(), None))
    torch.cuda.synchronize()
    assert _capi.status_read_and_clear() != 0
    big = torch.zeros(1, dtype=torch.float64, device="cuda")
    with pytest.raises(_capi.FvxError):
        _capi.check(lib.fvx_lu_solve_batched(1, 4096, big.data_ptr(), big.data_ptr(), None))


@pytest.mark.parametrize("free,loads", [(True, "kj"), (False, "bernoulli"), (True, "bernoulli")])
def test_free_ring_wake_and_bernoulli_loads(cuda, free, loads):
    """Free ring wake (every kept vertex moves with the induced velocity) and
    the unsteady Bernoulli loads of newton_pc/adapters/flap.py:357-401 on the
    three-surface configuration, against the oracle (prescribed particles)."""
    cfg = flapping_aircraft(n_keep=4, flapping="both", free_vpm=False, free_ring_wake=free,
                            loads=loads)
    g, o = _run(cfg, 10)
    assert _hist_err(g.cl, o.cl) < 1e-10
    if loads == "kj":
        assert _hist_err(g.cdi, o.cdi) < 1e-10
    else:
        assert np.abs(np.array(g.cdi) - np.array(o.cdi)).max() < 1e-10 * np.abs(o.cl).max()
    nv = o.W.shape[0] * o.W.shape[1]
    W = g.W[g.cur][:nv].cpu().numpy()
    assert np.abs(W - o.W.reshape(-1, 3)).max() < 1e-10
    assert rel_err(g.field.positions, o.p_pos) < 1e-10
