"""GB300-native hydroelastic contact engine.

A drop-in for the contact-surface path of the MuJoCo contact-surfaces plugin
(ubi-agni/mujoco_contact_surfaces): LBVH broadphase, element clipping,
pressure quadrature with Hunt-Crossley damping and regularised friction,
per-pair wrenches and flat tactile taxel binning as sm_103a kernels behind
the C ABI in include/hc/hc.h.
"""
from . import _lib
from ._lib import HCError, load
from .engine import Engine

__all__ = ["Engine", "HCError", "load", "_lib"]
