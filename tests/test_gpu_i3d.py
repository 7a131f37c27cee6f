"""The particledem C++ interface (cuda_addon/particledem.cuh:11-26) called the
way a caller compiled against the reference binds to it: by its C++ names,
with the i3d container types laid out as inshape3dcore/grid/uniformgrid.h
declares them (here as ctypes structures; the layouts are checked against
the reference's own header in test_reference_headers.py).

cuda_init builds the reference's jittered lattice (srand(1973) / rand());
then 20 steps of the particledem loop -- calcHash, sortParticles,
reorderDataAndFindCellStart, evalForces, integrateSystem -- each against the
oracle on the same input, bit for bit (the oracle with the GPU's fused
arithmetic)."""
import ctypes as C

import numpy as np
import pytest

from fcdem_testutil import assert_same_floats, check_cell_tables

pytestmark = pytest.mark.gpu


class Vec3(C.Structure):
    _fields_ = [("x", C.c_float), ("y", C.c_float), ("z", C.c_float)]


class SimulationParameters(C.Structure):
    _fields_ = [(n, C.c_float) for n in ("spring_", "damping_", "shear_", "attraction_",
                                         "boundaryDamping_", "globalDamping_",
                                         "particleRadius_", "timeStep_")] + \
               [("origin_", Vec3), ("cellSize_", Vec3), ("gravity_", Vec3)] + \
               [(n, C.c_uint) for n in ("gridx_", "gridy_", "gridz_", "numParticles_")]


class HashGrid(C.Structure):
    _fields_ = [("size_", C.c_uint), ("numCells_", C.c_uint),
                ("hashEntries_", C.c_void_p), ("particleIndices_", C.c_void_p),
                ("cellStart_", C.c_void_p), ("cellEnd_", C.c_void_p),
                ("gridx_", C.c_uint), ("gridy_", C.c_uint), ("gridz_", C.c_uint),
                ("cellSize_", Vec3), ("origin_", Vec3)]


class ParticleWorld(C.Structure):
    _fields_ = [("params_", C.POINTER(SimulationParameters)), ("pos_", C.c_void_p),
                ("vel_", C.c_void_p), ("sortedPos_", C.c_void_p), ("sortedVel_", C.c_void_p),
                ("size_", C.c_int)]


HG, PW = "RN3i3d8HashGridIfLi0EEE", "RNS_13ParticleWorldIfLi0EEE"
NAMES = {
    "cuda_init": f"_Z9cuda_init{HG}{PW}RPNS_20SimulationParametersIfEE",
    "cuda_clean": "_Z10cuda_cleanv",
    "calcHash": f"_Z8calcHash{HG}{PW}",
    "sortParticles": f"_Z13sortParticles{HG}",
    "reorder": f"_Z27reorderDataAndFindCellStart{HG}{PW}",
    "evalForces": f"_Z10evalForces{HG}{PW}",
    "integrateSystem": "_Z15integrateSystemPfS_fj",
}


def _fn(lib, key, args):
    f = getattr(lib, NAMES[key])
    f.argtypes = args
    f.restype = None
    return f


def test_particledem_interface_steps_match_oracle():
    from fullc0ntact_gb300 import dem
    from oracle import oracle as O
    lib = dem.lib
    n, r, g, dt = 4096, 1.0 / 64.0, 64, 0.5
    sp = SimulationParameters(spring_=0.5, damping_=0.02, shear_=0.1, attraction_=0.0,
                              boundaryDamping_=-0.5, globalDamping_=1.0, particleRadius_=r,
                              timeStep_=dt, origin_=Vec3(-1.0, -1.0, -1.0),
                              cellSize_=Vec3(2 * r, 2 * r, 2 * r),
                              gravity_=Vec3(0.0, 0.0, -3e-4), gridx_=g, gridy_=g, gridz_=g,
                              numParticles_=n)
    hg = HashGrid(size_=n)
    pw = ParticleWorld(params_=C.pointer(sp), size_=n)
    dev_params = C.c_void_p()
    P_hg, P_pw = C.POINTER(HashGrid), C.POINTER(ParticleWorld)
    _fn(lib, "cuda_init", [P_hg, P_pw, C.POINTER(C.c_void_p)])(C.byref(hg), C.byref(pw),
                                                                C.byref(dev_params))
    dem.check("cuda_init")
    assert hg.numCells_ == g ** 3 and abs(hg.cellSize_.x - 2 * r) == 0.0 and dev_params.value

    def fetch(ptr, count, dtype):
        a = np.empty(count, dtype)
        lib.copyArrayFromDevice(a.ctypes.data, ptr, None, a.nbytes)
        return a

    # the reference's lattice: side ceil(n^(1/3)), spacing 2r, jitter 0.01 r
    libc = C.CDLL(None)
    libc.rand.restype = C.c_int
    libc.srand(1973)
    rand_max = 2147483647.0
    s = int(np.ceil(np.float32(n) ** np.float32(1.0 / 3.0)))
    want = np.zeros((n, 4), np.float32)
    for i in range(n):
        x, y, z = i % s, (i // s) % s, i // (s * s)
        for k, c in enumerate((x, y, z)):
            u = np.float32(libc.rand() / rand_max)
            want[i, k] = np.float32(2 * r) * c + np.float32(r) - 1.0 + (u * 2.0 - 1.0) * np.float32(0.01 * r)
        want[i, 3] = 1.0
    pos0 = fetch(pw.pos_, 4 * n, np.float32).reshape(n, 4)
    np.testing.assert_allclose(pos0, want, rtol=0, atol=1e-6)

    calc = _fn(lib, "calcHash", [P_hg, P_pw])
    sort = _fn(lib, "sortParticles", [P_hg])
    reorder = _fn(lib, "reorder", [P_hg, P_pw])
    forces = _fn(lib, "evalForces", [P_hg, P_pw])
    integrate = _fn(lib, "integrateSystem", [C.c_void_p, C.c_void_p, C.c_float, C.c_uint])
    P = O.SimParams()
    P.gravity[:] = [0.0, 0.0, -3e-4]
    P.globalDamping = 1.0
    P.particleRadius = r
    P.gridSize[:] = [g, g, g]
    P.numCells = g ** 3
    P.worldOrigin[:] = [-1.0, -1.0, -1.0]
    P.cellSize[:] = [2 * r] * 3
    P.spring, P.damping, P.shear, P.attraction, P.boundaryDamping = 0.5, 0.02, 0.1, 0.0, -0.5
    rng = np.random.default_rng(3)
    vel = (rng.uniform(-0.01, 0.01, (n, 4)) * np.array([1, 1, 1, 0])).astype(np.float32)
    lib.copyArrayToDevice(pw.vel_, vel.ctypes.data, 0, vel.nbytes)  # a moving start
    pos = pos0.copy()
    with O.gpu_arithmetic():
        for step in range(20):
            calc(C.byref(hg), C.byref(pw))
            sort(C.byref(hg))
            reorder(C.byref(hg), C.byref(pw))
            forces(C.byref(hg), C.byref(pw))
            integrate(pw.pos_, pw.vel_, dt, n)
            dem.check(f"particledem step {step}")
            h, x = O.calc_hash(P, pos)
            hs, xs = O.sort_pairs(h, x)
            cs, ce, spos, svel = O.reorder(hs, xs, pos, vel, P.numCells)
            nv = O.collide(P, spos, svel, xs, cs, ce, False, False)
            O.integrate(P, pos, nv, dt)
            vel = nv
            np.testing.assert_array_equal(fetch(hg.hashEntries_, n, np.uint32), hs)
            np.testing.assert_array_equal(fetch(hg.particleIndices_, n, np.uint32), xs)
            check_cell_tables(fetch(hg.cellStart_, g ** 3, np.uint32),
                              fetch(hg.cellEnd_, g ** 3, np.uint32), cs, ce)
            assert_same_floats(fetch(pw.pos_, 4 * n, np.float32).reshape(n, 4), pos)
            assert_same_floats(fetch(pw.vel_, 4 * n, np.float32).reshape(n, 4)[:, :3],
                               vel[:, :3])
    assert np.count_nonzero(np.any(vel[:, :3] != 0, axis=1)) == n
    _fn(lib, "cuda_clean", [])()
    for a in ("hashEntries_", "particleIndices_", "cellStart_", "cellEnd_"):
        lib.freeArray(getattr(hg, a))
    for a in ("pos_", "vel_", "sortedPos_", "sortedVel_"):
        lib.freeArray(getattr(pw, a))
    dem.check("clean")
