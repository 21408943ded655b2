"""ibgb300: GB300-native immersed-boundary projection (CNAB) step.

Drop-in for the stream-function / CNAB path of ImmersedBoundary.jl: the reference's
problem / fluid / body / scheme constructors and its ``solve`` / ``advance!`` entry points,
backed by ``libibgb300.so`` (hand-written CUDA for sm_103a; see ``include/ibgb300.h``).
"""
from .api import *  # noqa: F401,F403
from .api import __all__ as _api_all
from . import workloads  # noqa: F401
from ._lib import IBError, load as load_library  # noqa: F401

__all__ = list(_api_all) + ["workloads", "IBError", "load_library"]
