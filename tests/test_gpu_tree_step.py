"""The treecode inside the particle integrator and the hybrid step: CL / CDi
of the heaving wing with treecode self-sweeps stay within 1e-4 of the FP64
direct step (the spec CL accuracy bar)."""
import numpy as np
import pytest

from fluxvortex_gb300.geometry import heaving_wing
from fluxvortex_gb300.hybrid import HybridStep

pytestmark = pytest.mark.gpu


def test_hybrid_with_tree_cl_within_1e4(cuda):
    steps = 24
    ref = HybridStep(heaving_wing(n_keep=4, free_vpm=True, stretch=True), precision="f64")
    cfg = heaving_wing(n_keep=4, free_vpm=True, stretch=True, far_field="tree")
    tre = HybridStep(cfg, precision="f32c")
    tre.field.tree.leaf_target = 16
    for _ in range(steps):
        ref.step()
        tre.step()
    cl_r, cl_t = ref.cl, tre.cl
    assert np.max(np.abs(cl_t - cl_r)) / np.max(np.abs(cl_r)) < 1e-4
    assert tre.field.np == ref.field.np > 0
