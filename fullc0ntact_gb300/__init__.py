"""fullc0ntact_gb300 -- GB300-native (sm_103a) particle-DEM step of
FullC0ntact behind the reference's particleSystem C-ABI.

The compute path is libfcdem.so (hand-written CUDA, built in-tree by
``fullc0ntact_gb300.build``); importing the package without it raises.
"""
from .params import SimParams, make_params  # noqa: F401
from . import _native  # noqa: F401  (raises ImportError without libfcdem.so)

__all__ = ["SimParams", "make_params"]
