"""libfcdem.so loads, exports every function include/*.h declares, and keeps
the reference's SimParams layout.  No compute calls (no GPU needed)."""
import ctypes as C
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


# C++ interfaces (exported under mangled names): checked separately
CPP_HEADERS = {"fcdem_i3d.h"}


def declared_functions():
    names = set()
    for f in os.listdir(os.path.join(ROOT, "include")):
        if not f.endswith(".h") or f in CPP_HEADERS:
            continue
        text = open(os.path.join(ROOT, "include", f)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        # the C++ class body is not part of the C-ABI
        text = re.sub(r"#ifdef __cplusplus\s*namespace.*?extern \"C\" \{", "", text, flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w \*]*?\b(\w+)\s*\([^;{]*\)\s*;", text, flags=re.M):
            names.add(m.group(1))
    names.discard("if")
    return sorted(names)


def test_library_exports_every_declared_function():
    from fullc0ntact_gb300 import _native
    decl = declared_functions()
    assert len(decl) >= 30
    missing = [n for n in decl if not hasattr(_native.lib, n)]
    assert not missing, missing
    out = subprocess.run(["nm", "-D", "--defined-only", _native.LIB_PATH],
                         capture_output=True, text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if line.strip()}
    assert not [n for n in decl if n not in exported]


def test_particledem_cpp_functions_exported():
    """The particledem C++ interface (cuda_addon/particledem.cuh:11-26) on the
    i3d types, exported under its C++ names."""
    from fullc0ntact_gb300 import _native
    out = subprocess.run(["nm", "-DC", "--defined-only", _native.LIB_PATH],
                         capture_output=True, text=True, check=True).stdout
    for sig in ["cuda_init(i3d::HashGrid<float, 0>&, i3d::ParticleWorld<float, 0>&, "
                "i3d::SimulationParameters<float>*&)", "cuda_clean()",
                "calcHash(i3d::HashGrid<float, 0>&, i3d::ParticleWorld<float, 0>&)",
                "reorderDataAndFindCellStart(i3d::HashGrid<float, 0>&, "
                "i3d::ParticleWorld<float, 0>&)",
                "evalForces(i3d::HashGrid<float, 0>&, i3d::ParticleWorld<float, 0>&)",
                "sortParticles(i3d::HashGrid<float, 0>&)",
                "integrateSystem(float*, float*, float, unsigned int)"]:
        assert sig in out, sig


def test_reference_entry_points_present():
    """The names of cuda_addon/particleSystem.cuh:12-63."""
    from fullc0ntact_gb300 import _native
    for n in ["cudaInit", "allocateArray", "freeArray", "threadSync", "copyArrayFromDevice",
              "copyArrayToDevice", "registerGLBufferObject", "unregisterGLBufferObject",
              "mapGLBufferObject", "unmapGLBufferObject", "setParameters", "integrateSystem",
              "calcHash", "reorderDataAndFindCellStart", "collide", "sortParticles"]:
        assert hasattr(_native.lib, n), n


def test_simparams_layout():
    """Offsets of cuda_addon/particles_kernel.cuh:27-48 (sizeof 104)."""
    from fullc0ntact_gb300.params import OFFSETS, SimParams
    assert C.sizeof(SimParams) == 104 and C.alignment(SimParams) == 4
    expect = dict(colliderPos=0, colliderRadius=12, gravity=16, globalDamping=28,
                  particleRadius=32, gridSize=36, numCells=48, worldOrigin=52, cellSize=64,
                  numBodies=76, maxParticlesPerCell=80, spring=84, damping=88, shear=92,
                  attraction=96, boundaryDamping=100)
    assert OFFSETS == expect


def test_simparams_matches_reference_header_layout():
    """The C header's struct, compiled, has the same offsets."""
    src = r'''
#include <stddef.h>
#include <stdio.h>
#include "fcdem.h"
int main(void){ printf("%zu %zu %zu %zu %zu\n", sizeof(SimParams), offsetof(SimParams, gridSize),
  offsetof(SimParams, worldOrigin), offsetof(SimParams, numBodies), offsetof(SimParams, boundaryDamping));
  return 0; }'''
    import tempfile
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "t.c")
        open(c, "w").write(src)
        exe = os.path.join(d, "t")
        subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), c, "-o", exe], check=True)
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()
    assert out == ["104", "36", "52", "76", "100"]


def test_error_strings_and_version():
    from fullc0ntact_gb300 import _native
    assert b"sm_103a" in _native.lib.fcdemVersion()
    for code in range(8):
        assert _native.lib.fcdemGetErrorString(code)


def test_product_does_not_reference_oracle():
    """The product package never imports or loads the oracle."""
    pkg = os.path.join(ROOT, "fullc0ntact_gb300")
    for dirpath, _, files in os.walk(pkg):
        for f in files:
            if f.endswith((".py", ".cu", ".cuh", ".cpp", ".h")):
                text = open(os.path.join(dirpath, f)).read()
                assert "oracle" not in text.replace("the oracle", ""), f
