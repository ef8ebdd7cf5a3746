"""patch()/unpatch() semantics of warp_patch.py:25-71 on a stand-in module
(PteraSoftware is a third-party package; the stand-in holds the oracle's
functions as the 'originals').  CPU only: no kernel is called."""
import types

from oracle import oracle as O
from fluxvortex_gb300 import aerodynamics, patch as P


def _standin():
    m = types.ModuleType("pterasoftware_standin_aerodynamics_functions")
    for name, fn in O.PS_FUNCTIONS.items():
        setattr(m, name, fn)
    return m


def test_patch_swaps_all_five_and_unpatch_restores(capsys):
    m = _standin()
    P.patch(module=m)
    try:
        assert P.is_active()
        for name in aerodynamics.PS_FUNCTION_NAMES:
            assert getattr(m, name) is getattr(aerodynamics, name)
        assert "GPU acceleration active" in capsys.readouterr().out
        P.patch(module=m)            # idempotent, silent
        assert capsys.readouterr().out == ""
    finally:
        P.unpatch()
    assert not P.is_active()
    for name, fn in O.PS_FUNCTIONS.items():
        assert getattr(m, name) is fn
    assert "Restored" in capsys.readouterr().out
    P.unpatch()                      # idempotent, silent
    assert capsys.readouterr().out == ""


def test_originals_saved_once():
    m = _standin()
    P.patch(module=m)
    P.unpatch()
    P.patch(module=m)
    P.unpatch()
    for name, fn in O.PS_FUNCTIONS.items():
        assert getattr(m, name) is fn


def test_signatures_match_reference_call_forms():
    import inspect
    ring = inspect.signature(aerodynamics.collapsed_velocities_from_ring_vortices)
    assert list(ring.parameters)[-3:] == ["singularity_counts", "ages", "nu"]
    assert ring.parameters["ages"].default is None and ring.parameters["nu"].default == 0.0
    hs = inspect.signature(aerodynamics.expanded_velocities_from_horseshoe_vortices)
    assert list(hs.parameters)[-2:] == ["singularity_counts", "nu"]
    assert len(ring.parameters) == 10 and len(hs.parameters) == 9
