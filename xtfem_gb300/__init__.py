"""GB300-native implementation of XTFEM's iterative space-time solve path.

The compute path lives in libxtfem_gb300.so (hand-written CUDA for sm_103a
behind a C ABI, include/xtfem_gb300.h); this package is its Python host
interface.  See api.py for the entry points.
"""
from ._lib import LIB_PATH, XtError, lib
from .api import *  # noqa: F401,F403
from .api import __all__ as _api_all

__all__ = ["LIB_PATH", "XtError", "lib", *_api_all]
__version__ = "0.1.0"
