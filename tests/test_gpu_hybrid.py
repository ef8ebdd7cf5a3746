"""Device hybrid panel-particle step against the oracle's restatement of the
reference's HybridSolver step (oracle/hybrid.py).  FP64: CL / CDi histories
within 1e-10 of the largest |CL| (the spec bar on the CL/CDi time
history); strengths and particle states within 1e-10 relative.  FP32
compensated particle sweeps: CL within 1e-4."""
import numpy as np
import pytest

from fluxvortex_gb300.geometry import heaving_wing, static_wing
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
