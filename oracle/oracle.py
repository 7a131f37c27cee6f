"""ctypes bindings of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this module: the CUDA kernels of ``fullc0ntact_gb300``
are tested against it; it is never part of the product path.

Three libraries are wrapped:

* ``_build/libfcdem_oracle.so`` -- the C restatement of the reference's
  particle-DEM step (``fcdem_oracle.c``), built on every machine.
* ``_ref/libfcref_host.so`` -- the reference's own ``particles_kernel.cu``
  compiled as host code (``ref_harness/refhost.cpp``); only where the
  reference tree was present at build time.
* ``_build/libfcref_gpu_loader.so`` + ``_ref/fcref_kernels.cubin`` -- the
  reference's kernels compiled for sm_103a and launched on the GPU.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF = os.path.join(HERE, "_ref")

_u32p = np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")
_f32p = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")

_lock = threading.Lock()
_libs: dict = {}


class SimParams(C.Structure):
    """The 104-byte parameter block of cuda_addon/particles_kernel.cuh:27-48."""

    _fields_ = [
        ("colliderPos", C.c_float * 3),
        ("colliderRadius", C.c_float),
        ("gravity", C.c_float * 3),
        ("globalDamping", C.c_float),
        ("particleRadius", C.c_float),
        ("gridSize", C.c_uint * 3),
        ("numCells", C.c_uint),
        ("worldOrigin", C.c_float * 3),
        ("cellSize", C.c_float * 3),
        ("numBodies", C.c_uint),
        ("maxParticlesPerCell", C.c_uint),
        ("spring", C.c_float),
        ("damping", C.c_float),
        ("shear", C.c_float),
        ("attraction", C.c_float),
        ("boundaryDamping", C.c_float),
    ]


assert C.sizeof(SimParams) == 104


class DistMap(C.Structure):
    _fields_ = [
        ("vmin", C.c_float * 3),
        ("vmax", C.c_float * 3),
        ("cellSize", C.c_float),
        ("cells", C.c_int * 3),
        ("distance", C.c_void_p),
        ("contactPoints", C.c_void_p),
    ]


def build(with_ref: bool = True) -> None:
    """Builds the oracle libraries (and the reference builds when possible)."""
    targets = ["all"] + (["ref"] if with_ref else [])
    subprocess.run(["make", "-s", "-C", HERE] + targets, check=True)


def _load(name: str, path: str):
    with _lock:
        if name not in _libs:
            if not os.path.exists(path):
                build(with_ref=False)
            _libs[name] = C.CDLL(path)
        return _libs[name]


def lib():
    L = _load("oracle", os.path.join(BUILD, "libfcdem_oracle.so"))
    if not getattr(L, "_typed", False):
        P = C.POINTER(SimParams)
        L.orc_integrate.argtypes = [P, _f32p, _f32p, C.c_float, C.c_uint, C.c_int]
        L.orc_calc_hash.argtypes = [P, _u32p, _u32p, _f32p, C.c_uint]
        L.orc_sort_pairs.argtypes = [_u32p, _u32p, C.c_uint]
        L.orc_reorder.argtypes = [_u32p, _u32p, _f32p, _f32p, _u32p, _u32p,
                                  _f32p, _f32p, C.c_uint, C.c_uint]
        L.orc_collide.argtypes = [P, _f32p, C.c_void_p, _f32p, _f32p, _u32p,
                                  _u32p, _u32p, C.c_uint, C.c_int, C.c_int, C.c_int]
        L.orc_collide_f64.argtypes = [P, _f64p, _f32p, _f32p, _u32p, _u32p,
                                      _u32p, C.c_uint, C.c_int, C.c_int, C.c_int]
        L.orc_update.argtypes = [P, C.c_float, _f32p, _f32p, _f32p, _f32p, _u32p,
                                 _u32p, _u32p, _u32p, C.c_uint, C.c_int, C.c_int]
        L.orc_distmap_query.argtypes = [C.POINTER(DistMap), _f32p, C.POINTER(C.c_float), _f32p]
        L.orc_integrate_distmap.argtypes = [P, C.POINTER(DistMap), _f32p, _f32p,
                                            C.c_float, C.c_uint, C.c_int]
        L.orc_set_gpu_arithmetic.argtypes = [C.c_int]
        L.orc_set_gpu_arithmetic.restype = None
        L.orc_integrate_box.argtypes = [P, _f32p, _f32p, _f32p, _f32p, C.c_float, C.c_uint,
                                        C.c_int]
        L.orc_batch_obstacle_integrate.argtypes = [P, _f32p, _f32p, C.c_void_p, _f32p, _f32p,
                                                   C.c_float, C.c_uint, C.c_int,
                                                   C.POINTER(C.c_uint)]
        for f in ("orc_integrate", "orc_calc_hash", "orc_sort_pairs", "orc_reorder",
                  "orc_collide", "orc_collide_f64", "orc_update", "orc_distmap_query",
                  "orc_integrate_distmap", "orc_integrate_box",
                  "orc_batch_obstacle_integrate"):
            getattr(L, f).restype = None
        L._typed = True
    return L


def scenegen():
    """The seeded scene generators built from the product's generator source
    as a host-only library (_build/libscenegen.so), for code that must build
    the benchmark's scenes without loading the GPU library."""
    return _load("scenegen", os.path.join(BUILD, "libscenegen.so"))


def ref_host_available() -> bool:
    return os.path.exists(os.path.join(REF, "libfcref_host.so"))


def ref_host():
    """The reference's own kernels built as host code (None if not built)."""
    path = os.path.join(REF, "libfcref_host.so")
    if not os.path.exists(path):
        return None
    L = _load("ref_host", path)
    if not getattr(L, "_typed", False):
        L.fcref_sizeof_simparams.restype = C.c_uint
        L.fcref_setParameters.argtypes = [C.POINTER(SimParams)]
        L.fcref_integrateSystem.argtypes = [_f32p, _f32p, C.c_float, C.c_uint]
        L.fcref_calcHash.argtypes = [_u32p, _u32p, _f32p, C.c_int]
        L.fcref_sortParticles.argtypes = [_u32p, _u32p, C.c_uint]
        L.fcref_reorderDataAndFindCellStart.argtypes = [
            _u32p, _u32p, _f32p, _f32p, _u32p, _u32p, _f32p, _f32p, C.c_uint, C.c_uint]
        L.fcref_collide.argtypes = [_f32p, _f32p, _f32p, _u32p, _u32p, _u32p,
                                    C.c_uint, C.c_uint]
        for f in ("fcref_setParameters", "fcref_integrateSystem", "fcref_calcHash",
                  "fcref_sortParticles", "fcref_reorderDataAndFindCellStart",
                  "fcref_collide"):
            getattr(L, f).restype = None
        L._typed = True
    return L


def ref_gpu():
    """The reference's kernels on the GPU (None when the cubin is absent).

    Raises RuntimeError when the cubin exists but cannot be loaded."""
    cubin = os.path.join(REF, "fcref_kernels.cubin")
    if not os.path.exists(cubin):
        return None
    L = _load("ref_gpu", os.path.join(BUILD, "libfcref_gpu_loader.so"))
    if not getattr(L, "_typed", False):
        L.fcrefgpu_load.argtypes = [C.c_char_p]
        L.fcrefgpu_set_parameters.argtypes = [C.POINTER(SimParams)]
        vp = C.c_void_p
        L.fcrefgpu_integrate.argtypes = [vp, vp, C.c_float, C.c_uint, vp]
        L.fcrefgpu_calc_hash.argtypes = [vp, vp, vp, C.c_uint, vp]
        L.fcrefgpu_reorder.argtypes = [vp] * 8 + [C.c_uint, C.c_uint, vp]
        L.fcrefgpu_collide.argtypes = [vp] * 6 + [C.c_uint, vp]
        rc = L.fcrefgpu_load(cubin.encode())
        if rc != 0:
            raise RuntimeError(f"loading the reference cubin failed (code {rc})")
        L._typed = True
    return L


def ref_thrust_sort():
    """thrust::sort_by_key on device arrays, as the reference's sortParticles
    issues it (particleSystem.cu:265-270); None when not built."""
    path = os.path.join(BUILD, "libfcref_thrust_sort.so")
    if not os.path.exists(path):
        return None
    L = _load("ref_thrust_sort", path)
    if not getattr(L, "_typed", False):
        L.fcrefgpu_sort_by_key.argtypes = [C.c_void_p, C.c_void_p, C.c_uint]
        L.fcrefgpu_sort_by_key.restype = C.c_int
        L._typed = True
    return L


def ref_distmap():
    """The reference's own distance-map query and boundary response built as
    host code (None if not built)."""
    path = os.path.join(REF, "libfcref_distmap.so")
    if not os.path.exists(path):
        return None
    L = _load("ref_distmap", path)
    if not getattr(L, "_typed", False):
        L.fcref_distmap_query.argtypes = [_f32p, _f32p, _f32p, _f32p, _f32p, C.c_float,
                                          np.ctypeslib.ndpointer(dtype=np.int32,
                                                                 flags="C_CONTIGUOUS"),
                                          _f32p, C.c_int, _f32p, _f32p]
        L.fcref_um_integrate.argtypes = [_f32p, _f32p, _f32p, _f32p, _f32p, _f32p, C.c_float,
                                         np.ctypeslib.ndpointer(dtype=np.int32,
                                                                flags="C_CONTIGUOUS"),
                                         _f32p, _f32p, C.c_int, _f32p, C.c_float, C.c_float,
                                         C.c_float, C.c_float]
        L.fcref_distmap_query.restype = None
        L.fcref_um_integrate.restype = None
        L._typed = True
    return L


class gpu_arithmetic:
    """Context manager: the oracle evaluates with the products nvcc contracts
    fused (orc_set_gpu_arithmetic), the arithmetic the GPU kernels spell out;
    on exit back to the host arithmetic of the reference's host build."""

    def __enter__(self):
        lib().orc_set_gpu_arithmetic(1)
        return self

    def __exit__(self, *exc):
        lib().orc_set_gpu_arithmetic(0)
        return False


def lattice_coords(vmin, cell_size, cells):
    """Vertex coordinates vmin + i*cellSize in float, vertex (i,j,k) at
    k*(cx+1)*(cy+1) + j*(cx+1) + i (distancemap.cpp:214-226)."""
    cs = np.float32(cell_size)
    ax = [np.float32(vmin[k]) + np.arange(cells[k] + 1, dtype=np.float32) * cs for k in range(3)]
    z, y, x = np.meshgrid(ax[2], ax[1], ax[0], indexing="ij")
    return np.ascontiguousarray(np.stack([x, y, z], axis=-1).reshape(-1, 3).astype(np.float32))


# ---------------------------------------------------------------------------
# numpy-level helpers


def integrate(P, pos, vel, dt, radius_from_w=False):
    lib().orc_integrate(C.byref(P), pos, vel, dt, pos.shape[0], int(radius_from_w))


def calc_hash(P, pos):
    n = pos.shape[0]
    h = np.empty(n, np.uint32)
    x = np.empty(n, np.uint32)
    lib().orc_calc_hash(C.byref(P), h, x, np.ascontiguousarray(pos), n)
    return h, x


def sort_pairs(keys, vals):
    k = keys.copy()
    v = vals.copy()
    lib().orc_sort_pairs(k, v, k.shape[0])
    return k, v


def reorder(hash_sorted, index_sorted, pos, vel, num_cells, cell_end_init=None):
    n = pos.shape[0]
    cs = np.empty(num_cells, np.uint32)
    ce = (np.full(num_cells, 0xFFFFFFFF, np.uint32) if cell_end_init is None
          else cell_end_init.copy())
    sp = np.empty_like(pos)
    sv = np.empty_like(vel)
    lib().orc_reorder(cs, ce, sp, sv, hash_sorted, index_sorted, pos, vel, n, num_cells)
    return cs, ce, sp, sv


def collide(P, sp, sv, index, cs, ce, radius_from_w=False, with_collider=True,
            nthreads=None, want_force=False):
    n = sp.shape[0]
    nv = np.zeros((n, 4), np.float32)
    force = np.zeros((n, 3), np.float32) if want_force else None
    nthreads = nthreads or os.cpu_count() or 1
    lib().orc_collide(C.byref(P), nv, force.ctypes.data if want_force else None,
                      sp, sv, index, cs, ce, n, int(radius_from_w),
                      int(with_collider), nthreads)
    return (nv, force) if want_force else nv


def collide_f64(P, sp, sv, index, cs, ce, radius_from_w=False, with_collider=True,
                nthreads=None):
    n = sp.shape[0]
    nv = np.zeros((n, 4), np.float64)
    lib().orc_collide_f64(C.byref(P), nv, sp, sv, index, cs, ce, n,
                          int(radius_from_w), int(with_collider),
                          nthreads or os.cpu_count() or 1)
    return nv


def step_stages(P, pos, vel, dt, radius_from_w=False, nthreads=None):
    """One ParticleSystem::update on copies; returns every intermediate."""
    pos = pos.copy()
    vel = vel.copy()
    integrate(P, pos, vel, dt, radius_from_w)
    h, x = calc_hash(P, pos)
    hs, xs = sort_pairs(h, x)
    cs, ce, sp, sv = reorder(hs, xs, pos, vel, P.numCells)
    nv = collide(P, sp, sv, xs, cs, ce, radius_from_w, True, nthreads)
    return dict(pos=pos, vel_in=vel, hash=h, index=x, hash_sorted=hs,
                index_sorted=xs, cellStart=cs, cellEnd=ce, sortedPos=sp,
                sortedVel=sv, newVel=nv)


def update(P, pos, vel, dt, steps=1, radius_from_w=False, nthreads=None):
    """`steps` full updates in place (pos, vel are (n, 4) float32)."""
    n = pos.shape[0]
    sp = np.empty_like(pos)
    sv = np.empty_like(vel)
    h = np.empty(n, np.uint32)
    x = np.empty(n, np.uint32)
    cs = np.empty(P.numCells, np.uint32)
    ce = np.full(P.numCells, 0xFFFFFFFF, np.uint32)
    L = lib()
    for _ in range(steps):
        L.orc_update(C.byref(P), dt, pos, vel, sp, sv, h, x, cs, ce, n,
                     int(radius_from_w), nthreads or os.cpu_count() or 1)


def distmap_struct(vmin, vmax, cell_size, cells, distance, contact_points):
    m = DistMap()
    m.vmin[:] = [float(v) for v in vmin]
    m.vmax[:] = [float(v) for v in vmax]
    m.cellSize = float(cell_size)
    m.cells[:] = [int(c) for c in cells]
    m.distance = distance.ctypes.data
    m.contactPoints = contact_points.ctypes.data
    m._keep = (distance, contact_points)
    return m


def distmap_query(m, q):
    d = C.c_float()
    cp = np.zeros(3, np.float32)
    lib().orc_distmap_query(C.byref(m), np.ascontiguousarray(q, np.float32),
                            C.byref(d), cp)
    return d.value, cp


def integrate_distmap(P, m, pos, vel, dt, radius_from_w=False):
    lib().orc_integrate_distmap(C.byref(P), C.byref(m), pos, vel, dt, pos.shape[0],
                                int(radius_from_w))


# ---------------------------------------------------------------------------
# batched scenes: each scene of a batch is one ParticleSystem in its own box


def _box(scene):
    lo = np.ascontiguousarray(scene.get("box_lo", (-1.0, -1.0, -1.0)), np.float32)
    hi = np.ascontiguousarray(scene.get("box_hi", (1.0, 1.0, 1.0)), np.float32)
    return lo, hi


def integrate_box(P, lo, hi, pos, vel, dt, radius_from_w=False):
    lib().orc_integrate_box(C.byref(P), np.ascontiguousarray(lo, np.float32),
                            np.ascontiguousarray(hi, np.float32), pos, vel, dt,
                            pos.shape[0], int(radius_from_w))


def batch_obstacle_integrate(P, lo, hi, m, pos, vel, dt, radius_from_w=False):
    """The obstacle integrate of a batched scene; m is a DistMap (or None).
    Returns the number of particles the map pushed out."""
    nc = C.c_uint(0)
    lib().orc_batch_obstacle_integrate(C.byref(P), np.ascontiguousarray(lo, np.float32),
                                       np.ascontiguousarray(hi, np.float32),
                                       C.cast(C.pointer(m), C.c_void_p) if m is not None
                                       else None, pos, vel, dt, pos.shape[0],
                                       int(radius_from_w), C.byref(nc))
    return int(nc.value)


def batch_scene_step(scene, m=None, obstacle=False, nthreads=None, pos=None, vel=None):
    """One update of one batched scene on copies of (pos, vel) (default: the
    scene's): the integrate in the scene's box (with the obstacle contact of
    map m when `obstacle`), calcHash, sortParticles, reorder, collide with
    the collider sphere (the batch step always applies it).  Returns every
    intermediate, as step_stages."""
    P = SimParams.from_buffer_copy(bytes(scene["params"]))
    w = bool(scene.get("radius_from_w", False))
    pos = (scene["pos"] if pos is None else pos).copy()
    vel = (scene["vel"] if vel is None else vel).copy()
    lo, hi = _box(scene)
    contacts = 0
    if obstacle:
        contacts = batch_obstacle_integrate(P, lo, hi, m, pos, vel, scene["dt"], w)
    else:
        integrate_box(P, lo, hi, pos, vel, scene["dt"], w)
    h, x = calc_hash(P, pos)
    hs, xs = sort_pairs(h, x)
    cs, ce, sp, sv = reorder(hs, xs, pos, vel, P.numCells)
    nv = collide(P, sp, sv, xs, cs, ce, w, True, nthreads)
    return dict(pos=pos, vel_in=vel, hash=h, index=x, hash_sorted=hs, index_sorted=xs,
                cellStart=cs, cellEnd=ce, sortedPos=sp, sortedVel=sv, newVel=nv,
                map_contacts=contacts)
