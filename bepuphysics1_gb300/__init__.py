"""GB300 velocity solver and integration step for BEPUphysics v1 scenes.

The solver path (ForceUpdater -> Solver -> PositionUpdater) runs as
hand-written sm_103a CUDA behind the C ABI in include/bepugpu.h; this package
is the Python host side over that ABI and the seeded scene source.
"""
from . import native
from .native import (ArgumentException, BepuError, InvalidOperationException, BODY_DTYPE, MANIFOLD_DTYPE,
                     JOINT_DTYPE, SETTINGS_DTYPE, CONTACT_DTYPE)

__all__ = ["native", "ArgumentException", "BepuError", "InvalidOperationException", "BODY_DTYPE",
           "MANIFOLD_DTYPE", "JOINT_DTYPE", "SETTINGS_DTYPE", "CONTACT_DTYPE"]
