"""GB300 (sm_103a) implementation of WumingPIC's particle-in-cell time step.

The compute path is the CUDA library ``_build/libwumingpic_gb300.so`` behind the
C ABI in ``include/wumingpic_gb300.h``; this package is its host-side mirror of
the reference's module interface (``pic2d.Pic2D``) plus the seeded synthetic
loader (``loader``).
"""
from .loader import Plasma2D, State2D, config_weibel2d, empty_state2d, load_weibel2d  # noqa: F401

__all__ = ["Plasma2D", "State2D", "config_weibel2d", "empty_state2d", "load_weibel2d", "Pic2D"]


def __getattr__(name):
    if name == "Pic2D":
        from .pic2d import Pic2D
        return Pic2D
    raise AttributeError(name)
