"""Loads libfcdem.so (the C-ABI library) and declares its entry points.

The library is built in-tree by ``fullc0ntact_gb300.build``.  There is no
fallback: when the library is missing or fails to load, importing this module
raises, so nothing can silently run a CPU path instead of the CUDA kernels.
"""
from __future__ import annotations

import ctypes as C
import os

from .params import SimParams

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libfcdem.so")

if not os.path.exists(LIB_PATH):
    raise ImportError(
        f"{LIB_PATH} is missing: build it with `python -m fullc0ntact_gb300.build` "
        "(nvcc for sm_103a is required; there is no CPU fallback)")

lib = C.CDLL(LIB_PATH)

vp = C.c_void_p
u32 = C.c_uint
P = C.POINTER(SimParams)

_SIGS = {
    # reference names (cuda_addon/particleSystem.cuh:12-63)
    "cudaInit": (None, [C.c_int, C.POINTER(C.c_char_p)]),
    "allocateArray": (None, [C.POINTER(vp), C.c_int]),
    "freeArray": (None, [vp]),
    "threadSync": (None, []),
    "copyArrayFromDevice": (None, [vp, vp, vp, C.c_int]),
    "copyArrayToDevice": (None, [vp, vp, C.c_int, C.c_int]),
    "registerGLBufferObject": (None, [u32, vp]),
    "unregisterGLBufferObject": (None, [vp]),
    "mapGLBufferObject": (vp, [vp]),
    "unmapGLBufferObject": (None, [vp]),
    "setParameters": (None, [P]),
    "integrateSystem": (None, [vp, vp, C.c_float, u32]),
    "calcHash": (None, [vp, vp, vp, C.c_int]),
    "sortParticles": (None, [vp, vp, u32]),
    "fcdemSortParticlesNoAlloc": (None, [vp, vp, u32]),
    "reorderDataAndFindCellStart": (None, [vp] * 8 + [u32, u32]),
    "collide": (None, [vp] * 6 + [u32, u32]),
    # extensions
    "fcdemGetLastError": (C.c_int, []),
    "fcdemGetErrorString": (C.c_char_p, [C.c_int]),
    "fcdemSetStream": (None, [vp]),
    "fcdemSetRadiusMode": (None, [C.c_int]),
    "fcdemVersion": (C.c_char_p, []),
    "fcdemSetCollidePath": (None, [C.c_int]),
    "fcdemSetCellCulling": (None, [C.c_int]),
    "fcdemSetCrowdPath": (None, [C.c_int]),
    "fcdemSetCellOrder": (None, [C.c_int]),
    "fcdemSetCrowdLimit": (None, [C.c_uint]),
    "fcdemSetUpdatePipeline": (None, [C.c_int]),
    "fcdemAutotuneSort": (C.c_int, [C.c_uint, C.c_uint, C.POINTER(C.c_float)]),
    "fcdemSetSortConfig": (C.c_int, [C.c_uint, C.c_int]),
    "fcdemSetSortWaitLimit": (None, [C.c_int]),
    "fcdemAutotuneCollide": (C.c_int, [vp] * 8 + [C.c_float, u32, u32, C.POINTER(C.c_float)]),
    "fcdemSetCollideConfig": (C.c_int, [C.c_int]),
    "fcdemGetCollideConfig": (C.c_int, [C.c_int, C.POINTER(C.c_uint), C.POINTER(C.c_uint),
                                        C.POINTER(C.c_int)]),
    "fcdemWriteVtkParticles": (C.c_int, [C.c_char_p, vp, vp, u32, C.c_float, C.c_int]),
    "fcdemWriteGPUParticleFile": (C.c_int, [vp, u32, C.c_char_p]),
}

for _name, (_res, _args) in _SIGS.items():
    _f = getattr(lib, _name)
    _f.restype = _res
    _f.argtypes = _args


class FcdemError(RuntimeError):
    pass


def check(what: str = "fcdem call") -> None:
    """Raises FcdemError if the library recorded an error (synchronises)."""
    code = lib.fcdemGetLastError()
    if code != 0:
        msg = lib.fcdemGetErrorString(code).decode()
        raise FcdemError(f"{what}: {msg} (code {code})")


def exported_symbols() -> list[str]:
    return list(_SIGS)
