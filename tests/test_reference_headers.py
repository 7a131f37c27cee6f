"""The drop-in boundary against the reference's own headers (CPU only; no
GPU call).  Skipped where the reference tree is absent; its path is the one
oracle/Makefile builds the reference's sources from (FCDEM_REFERENCE_TREE
overrides it).

* A program that includes cuda_addon/particles_kernel.cuh and
  particleSystem.cuh and this library's fcdem.h in one translation unit
  compiles (so every extern "C" declaration of fcdem.h agrees with the
  reference's), links against libfcdem.so and resolves all sixteen entry
  points.
* A program on the reference's i3d container types
  (inshape3dcore/grid/uniformgrid.h) links against the particledem C++
  functions of libfcdem.so (the mangled names match), and the member
  offsets of the three types equal those of fcdem_i3d.h's declarations."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ABI = os.path.join(ROOT, "tests", "abi")
LIBDIR = os.path.join(ROOT, "fullc0ntact_gb300", "_lib")
CUDA_INC = "/usr/local/cuda/include"


def _reference_tree():
    r = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "print-ref"],
                       capture_output=True, text=True)
    ref = r.stdout.strip()
    if r.returncode != 0 or not os.path.isdir(os.path.join(ref, "cuda_addon")):
        pytest.skip("reference tree not present")
    return ref


def _build_and_run(src, includes, tmp_path):
    from fullc0ntact_gb300 import build
    build.build()
    exe = str(tmp_path / (os.path.basename(src) + ".bin"))
    cmd = (["g++", "-std=c++17", "-O0", "-w", src, "-o", exe] +
           [f"-I{d}" for d in includes] +
           ["-L" + LIBDIR, "-lfcdem", "-Wl,-rpath," + LIBDIR,
            "-L/usr/local/cuda/lib64", "-Wl,-rpath,/usr/local/cuda/lib64"])
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    out = subprocess.run([exe], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    return out.stdout


def test_reference_c_interface_header_compiles_with_ours_and_links(tmp_path):
    ref = _reference_tree()
    out = _build_and_run(os.path.join(ABI, "ref_particlesystem_driver.cpp"),
                         [os.path.join(ref, "cuda_addon"), os.path.join(ROOT, "include"),
                          CUDA_INC], tmp_path)
    assert "resolved 16 of 16" in out


def test_reference_i3d_types_link_to_particledem_functions(tmp_path):
    ref = _reference_tree()
    dirs = []
    for top in ("math", "inshape3dcore", "util"):
        for d, _, _ in os.walk(os.path.join(ref, top)):
            dirs.append(d)
    theirs = _build_and_run(os.path.join(ABI, "ref_particledem_driver.cpp"),
                            dirs + [os.path.join(ROOT, "include"), CUDA_INC], tmp_path)
    ours = _build_and_run(os.path.join(ABI, "own_particledem_layout.cpp"),
                          [os.path.join(ROOT, "include")], tmp_path)
    assert "resolved 7 of 7" in theirs
    assert theirs == ours, (theirs, ours)
