"""fullc0ntact_gb300 -- GB300-native (sm_103a) particle-DEM step of
FullC0ntact behind the reference's particleSystem C-ABI.

The compute path is libfcdem.so (hand-written CUDA, built in-tree by
``fullc0ntact_gb300.build``).  The modules that call it (``dem``, ``scenes``)
load it through ``_native``, which raises ImportError when it is missing:
there is no CPU fallback.
"""
from .params import SimParams, make_params  # noqa: F401

__all__ = ["SimParams", "make_params"]
