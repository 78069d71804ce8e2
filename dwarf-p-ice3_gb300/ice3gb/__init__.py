"""ice3gb — GB300-native (sm_103a) FP64 ICE3 microphysics hot path.

Drop-in components mirroring the reference's callables
(maurinl26/dwarf-p-ice3):

* :class:`IceAdjust`   ~ ``IceAdjustJAX``   (src/ice3/jax/ice_adjust.py:40)
* :class:`RainIce`     ~ ``RainIceJAX``     (src/ice3/jax/rain_ice.py:20)
* :class:`Sedimentation` ~ ``sedimentation_stat`` (src/ice3/jax/stencils/sedimentation.py:58)

All compute runs in hand-written CUDA kernels behind the C ABI of
include/ice3gb.h (``libice3gb.so``); there is no CPU fallback.
"""
from .constants import build_table, ConstantsTable  # noqa: F401

__all__ = ["IceAdjust", "RainIce", "Sedimentation", "build_table", "ConstantsTable"]


def __getattr__(name):
    if name in ("IceAdjust", "RainIce", "Sedimentation", "Ice3Handle"):
        from . import components
        return getattr(components, name)
    raise AttributeError(name)
