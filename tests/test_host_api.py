"""Host-side pieces that need no GPU: the VTK particle writers, the C++
particledem interface header (compiles and links against libfcdem.so), the
scene generators, the collide configuration table."""
import ctypes as C
import os
import subprocess
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_vtk_writer_format(tmp_path):
    from fullc0ntact_gb300 import _native
    lib = _native.lib
    lib.fcdemWriteVtkParticles.argtypes = [C.c_char_p, C.c_void_p, C.c_void_p, C.c_uint,
                                           C.c_float, C.c_int]
    lib.fcdemWriteVtkParticles.restype = C.c_int
    pos = np.array([[0.5, -0.25, 1.0, 0.01], [0.0, 0.125, -0.5, 0.02]], np.float32)
    vel = np.array([[1.0, 2.0, 3.0, 0.0], [4.0, 5.0, 6.0, 0.0]], np.float32)
    path = str(tmp_path / "p.vtk")
    assert lib.fcdemWriteVtkParticles(path.encode(), pos.ctypes.data, vel.ctypes.data, 2,
                                      1.0 / 64.0, 1) == 0
    lines = open(path).read().splitlines()
    assert lines[:5] == ["# vtk DataFile Version 2.0", "Generated by fcdem-gb300", "ASCII",
                         "DATASET UNSTRUCTURED_GRID", "POINTS 2 double"]
    assert lines[5].split() == ["0.500000", "-0.250000", "1.000000"]
    i = lines.index("SCALARS radius double 1")
    assert [float(x) for x in lines[i + 2:i + 4]] == [0.01, 0.02]
    i = lines.index("SCALARS myid double 1")
    assert [float(x) for x in lines[i + 2:i + 4]] == [0.0, 1.0]
    assert "VECTORS velocity double" in lines
    assert lib.fcdemWriteVtkParticles(b"/nonexistent/dir/p.vtk", pos.ctypes.data, None, 2,
                                      0.1, 0) != 0


def test_gpu_particle_file_is_the_reference_format(tmp_path):
    """fcdemWriteGPUParticleFile writes the bytes of the reference's
    CVtkWriter::WriteGPUParticleFile (vtkwriter.cpp:3399-3452): its four
    header lines, "POINTS n double", each point as three %f fields and a
    trailing space, POINT_DATA, the radius 1/64 for every particle and the
    particle numbers as the "myid" scalar."""
    from fullc0ntact_gb300 import _native
    lib = _native.lib
    rng = np.random.default_rng(5)
    pos = rng.uniform(-1.0, 1.0, (37, 4)).astype(np.float32)
    path = str(tmp_path / "gpu.vtk")
    assert lib.fcdemWriteGPUParticleFile(pos.ctypes.data, 37, path.encode()) == 0
    want = ["# vtk DataFile Version 2.0", "Generated by InShape 2.x", "ASCII",
            "DATASET UNSTRUCTURED_GRID", "POINTS 37 double"]
    want += ["%f %f %f " % tuple(float(v) for v in p[:3]) for p in pos]
    want += ["POINT_DATA 37", "SCALARS radius double 1", "LOOKUP_TABLE default"]
    want += ["%f " % float(np.float32(1.0 / 64.0))] * 37
    want += ["SCALARS myid double 1", "LOOKUP_TABLE default"]
    want += ["%f " % float(i) for i in range(37)]
    assert open(path, "rb").read() == ("\n".join(want) + "\n").encode()
    assert lib.fcdemWriteGPUParticleFile(pos.ctypes.data, 37, b"/nonexistent/dir/p.vtk") != 0


def test_particledem_header_compiles_and_links():
    """A program on fcdem_i3d.h alone (the i3d container types declared there,
    no reference tree) resolves every particledem function of
    cuda_addon/particledem.cuh:11-26 in libfcdem.so."""
    from fullc0ntact_gb300 import _native
    src = r'''
#include "fcdem_i3d.h"
int main() {
  i3d::HashGrid<float, i3d::cpu> hg;
  i3d::ParticleWorld<float, i3d::cpu> pw;
  (void)hg; (void)pw;
  /* no GPU work: only check that every call resolves */
  void (*a)(i3d::HashGrid<float, i3d::cpu> &, i3d::ParticleWorld<float, i3d::cpu> &) = calcHash;
  void (*b)(i3d::HashGrid<float, i3d::cpu> &) = sortParticles;
  void (*c)(i3d::HashGrid<float, i3d::cpu> &, i3d::ParticleWorld<float, i3d::cpu> &) =
      reorderDataAndFindCellStart;
  void (*d)(i3d::HashGrid<float, i3d::cpu> &, i3d::ParticleWorld<float, i3d::cpu> &) = evalForces;
  void (*e)(float *, float *, float, unsigned int) = integrateSystem;
  void (*f)() = cuda_clean;
  return (a && b && c && d && e && f && cuda_init) ? 0 : 2;
}'''
    with tempfile.TemporaryDirectory() as tmp:
        cpp = os.path.join(tmp, "t.cpp")
        open(cpp, "w").write(src)
        exe = os.path.join(tmp, "t")
        libdir = os.path.dirname(_native.LIB_PATH)
        subprocess.run(["g++", "-std=c++17", "-I", os.path.join(ROOT, "include"), cpp, "-o", exe,
                        "-L", libdir, "-lfcdem", f"-Wl,-rpath,{libdir}"], check=True)
        assert subprocess.run([exe]).returncode == 0


def test_packing_has_no_overlaps_and_reaches_density():
    from fullc0ntact_gb300 import scenes
    sc = scenes.packed_scene(20000, grid=64)
    p = sc["pos"].astype(np.float64)
    r = p[:, 3]
    assert r.max() <= 2.0 / 512.0 + 1e-9 and r.min() > 0
    # brute force on a subset: no two spheres overlap
    idx = np.random.default_rng(0).choice(len(p), 2000, replace=False)
    d = np.linalg.norm(p[idx, None, :3] - p[None, :, :3], axis=2)
    rr = r[idx, None] + r[None, :]
    d[np.arange(2000), idx] = np.inf
    assert np.all(d >= rr * (1 - 1e-6))
    vf = (4.0 / 3.0 * np.pi * r ** 3).sum() / sc["box_side"] ** 3
    assert 0.28 <= vf <= 0.31


def test_scene_generators_are_deterministic():
    from fullc0ntact_gb300 import scenes
    a, b = scenes.lattice_scene(1000), scenes.lattice_scene(1000)
    np.testing.assert_array_equal(a["pos"], b["pos"])
    c, d = scenes.packed_scene(3000, grid=32), scenes.packed_scene(3000, grid=32)
    np.testing.assert_array_equal(c["pos"], d["pos"])


def test_collide_configuration_table():
    """The collide configurations the autotuner chooses from: 5 crowd limits x
    3 persistent-grid widths x row staging on/off, the default (512, 4 CTAs
    per SM, staged) among them.  Reading the table needs no GPU."""
    from fullc0ntact_gb300 import _native
    lib = _native.lib
    count = lib.fcdemSetCollideConfig(-1)
    assert count == 30
    seen = set()
    for k in range(count):
        lim, ctas, stage = C.c_uint(), C.c_uint(), C.c_int()
        assert lib.fcdemGetCollideConfig(k, C.byref(lim), C.byref(ctas), C.byref(stage)) == 0
        seen.add((lim.value, ctas.value, stage.value))
    assert len(seen) == 30 and (512, 4, 1) in seen
    assert {s[0] for s in seen} == {256, 384, 512, 768, 1024}
    assert {s[1] for s in seen} == {2, 4, 8}
