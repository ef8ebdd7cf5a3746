"""fluxvortex_gb300 -- GB300 (sm_103a) hybrid panel-particle vortex-induction path.

Drop-in for FLUXVortex's induction hot path:
  * ``fluxvortex_gb300.patch``        patch()/unpatch(): swap PteraSoftware's
                                      Biot-Savart functions (warp_patch.py)
  * ``fluxvortex_gb300.aerodynamics`` the five PS-signature functions
                                      (warp_kernels.py)
  * ``fluxvortex_gb300.kernel``       particle velocity / Jacobian (kernel.py)
  * ``fluxvortex_gb300.particles``    device-resident VortexParticleField
                                      (particles.py)

All compute runs in the C-ABI library ``_lib/libfluxvortex_gb300.so`` built
from ``csrc/`` (``python -m fluxvortex_gb300.build``).
"""
from . import _capi  # noqa: F401

__version__ = "0.1.0"


def library():
    """The loaded ctypes library (built on first use)."""
    return _capi.load()
