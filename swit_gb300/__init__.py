"""swit_gb300: GB300-native forward/adjoint wave-propagation engine behind SWIT's
toolbox/solver.py forward() and adjoint() calls.

Hand-written sm_103a CUDA kernels (swit_gb300/csrc) behind a C ABI
(include/swit_gb300.h), driven from Python through ctypes.
"""
from .engine import Engine, MultiEngine, damp_profile  # noqa: F401
from ._lib import SwitError  # noqa: F401

__all__ = ["Engine", "damp_profile", "SwitError"]
