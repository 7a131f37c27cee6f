"""Python face of libfcdem: the reference-named stages on torch device
tensors, a device-resident scene, and the ParticleSystem wrapper.

torch is used only to own device memory and streams; every computation is a
call into libfcdem.so through its C-ABI.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _native
from .params import SimParams

lib = _native.lib
check = _native.check


def _p(t: torch.Tensor) -> int:
    if not t.is_cuda:
        raise ValueError("libfcdem stages take CUDA tensors")
    if not t.is_contiguous():
        raise ValueError("libfcdem stages take contiguous tensors")
    return t.data_ptr()


# --- the five stages, reference names and argument order -------------------

def set_parameters(params: SimParams) -> None:
    lib.setParameters(C.byref(params))


def set_radius_mode(radius_from_w: bool) -> None:
    lib.fcdemSetRadiusMode(1 if radius_from_w else 0)


def set_stream(stream: torch.cuda.Stream | None) -> None:
    lib.fcdemSetStream(None if stream is None else stream.cuda_stream)


def integrate_system(pos, vel, dt: float, n: int) -> None:
    lib.integrateSystem(_p(pos), _p(vel), dt, n)


def calc_hash(hash_, index, pos, n: int) -> None:
    lib.calcHash(_p(hash_), _p(index), _p(pos), n)


def sort_particles(hash_, index, n: int) -> None:
    lib.sortParticles(_p(hash_), _p(index), n)


def reorder_data_and_find_cell_start(cell_start, cell_end, sorted_pos, sorted_vel,
                                     hash_, index, old_pos, old_vel, n: int,
                                     num_cells: int) -> None:
    lib.reorderDataAndFindCellStart(_p(cell_start), _p(cell_end), _p(sorted_pos),
                                    _p(sorted_vel), _p(hash_), _p(index), _p(old_pos),
                                    _p(old_vel), n, num_cells)


def collide(new_vel, sorted_pos, sorted_vel, index, cell_start, cell_end, n: int,
            num_cells: int) -> None:
    lib.collide(_p(new_vel), _p(sorted_pos), _p(sorted_vel), _p(index), _p(cell_start),
                _p(cell_end), n, num_cells)


lib.fcdemUpdate.argtypes = [C.c_void_p] * 8 + [C.c_float, C.c_uint, C.c_uint, C.c_uint]
lib.fcdemUpdate.restype = None


def update(pos, vel, sorted_pos, sorted_vel, hash_, index, cell_start, cell_end,
           dt: float, n: int, num_cells: int, steps: int = 1) -> None:
    lib.fcdemUpdate(_p(pos), _p(vel), _p(sorted_pos), _p(sorted_vel), _p(hash_),
                    _p(index), _p(cell_start), _p(cell_end), dt, n, num_cells, steps)


# --- device-resident scene -------------------------------------------------

class DeviceScene:
    """The work arrays of ParticleSystem (particleSystem.cpp:117-190) for one
    scene, as torch CUDA tensors."""

    def __init__(self, scene: dict, device: str | torch.device = "cuda"):
        self.params: SimParams = scene["params"].copy()
        self.radius_from_w = bool(scene.get("radius_from_w", False))
        self.dt = float(scene.get("dt", 0.5))
        self.n = int(scene["pos"].shape[0])
        self.num_cells = int(self.params.numCells)
        dev = torch.device(device)
        self.pos = torch.from_numpy(np.ascontiguousarray(scene["pos"])).to(dev)
        self.vel = torch.from_numpy(np.ascontiguousarray(scene["vel"])).to(dev)
        self.sorted_pos = torch.empty_like(self.pos)
        self.sorted_vel = torch.empty_like(self.vel)
        self.hash = torch.empty(self.n, dtype=torch.int32, device=dev)
        self.index = torch.empty(self.n, dtype=torch.int32, device=dev)
        self.cell_start = torch.empty(self.num_cells, dtype=torch.int32, device=dev)
        self.cell_end = torch.full((self.num_cells,), -1, dtype=torch.int32, device=dev)

    def activate(self) -> None:
        set_parameters(self.params)
        set_radius_mode(self.radius_from_w)

    def stages(self, dt: float | None = None) -> None:
        """One update as the reference issues it: five separate calls."""
        dt = self.dt if dt is None else dt
        self.activate()
        integrate_system(self.pos, self.vel, dt, self.n)
        calc_hash(self.hash, self.index, self.pos, self.n)
        sort_particles(self.hash, self.index, self.n)
        reorder_data_and_find_cell_start(self.cell_start, self.cell_end, self.sorted_pos,
                                         self.sorted_vel, self.hash, self.index, self.pos,
                                         self.vel, self.n, self.num_cells)
        collide(self.vel, self.sorted_pos, self.sorted_vel, self.index, self.cell_start,
                self.cell_end, self.n, self.num_cells)

    def update(self, steps: int = 1, dt: float | None = None) -> None:
        """`steps` updates through the fused fcdemUpdate."""
        dt = self.dt if dt is None else dt
        self.activate()
        update(self.pos, self.vel, self.sorted_pos, self.sorted_vel, self.hash,
               self.index, self.cell_start, self.cell_end, dt, self.n, self.num_cells,
               steps)

    def autotune_collide(self, dt: float | None = None) -> tuple[int, float]:
        """fcdemAutotuneCollide from this scene's state: the index of the
        fastest collide configuration (kept for later updates) and its step
        time in ms.  pos and vel are left as they were."""
        dt = self.dt if dt is None else dt
        self.activate()
        ms = C.c_float()
        k = lib.fcdemAutotuneCollide(_p(self.pos), _p(self.vel), _p(self.sorted_pos),
                                     _p(self.sorted_vel), _p(self.hash), _p(self.index),
                                     _p(self.cell_start), _p(self.cell_end), dt, self.n,
                                     self.num_cells, C.byref(ms))
        check("fcdemAutotuneCollide")
        return int(k), float(ms.value)


def u32(t: torch.Tensor) -> np.ndarray:
    """int32 device tensor -> uint32 host array (same bits)."""
    return t.cpu().numpy().view(np.uint32)


# --- ParticleSystem (C++ class behind a C wrapper) --------------------------

_PS_SIGS = {
    "fcdemPS_create": (C.c_void_p, [C.c_uint] * 4),
    "fcdemPS_destroy": (None, [C.c_void_p]),
    "fcdemPS_params": (C.POINTER(SimParams), [C.c_void_p]),
    "fcdemPS_update": (None, [C.c_void_p, C.c_float]),
    "fcdemPS_updateSteps": (None, [C.c_void_p, C.c_float, C.c_uint]),
    "fcdemPS_reset": (None, [C.c_void_p, C.c_int]),
    "fcdemPS_setArray": (None, [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_int]),
    "fcdemPS_getArray": (C.POINTER(C.c_float), [C.c_void_p, C.c_int]),
    "fcdemPS_dumpGrid": (C.c_uint, [C.c_void_p]),
    "fcdemPS_setFusedUpdate": (None, [C.c_void_p, C.c_int]),
    "fcdemPS_setRadiusFromW": (None, [C.c_void_p, C.c_int]),
    "fcdemPS_devicePos": (C.c_void_p, [C.c_void_p]),
    "fcdemPS_deviceVel": (C.c_void_p, [C.c_void_p]),
}
for _n, (_r, _a) in _PS_SIGS.items():
    getattr(lib, _n).restype = _r
    getattr(lib, _n).argtypes = _a


class ParticleSystem:
    """The reference's ParticleSystem (particleSystem.h:22-136), headless:
    constructor(numParticles, gridSize), update(dt), reset(config),
    getArray/setArray, the setters, dumpGrid."""

    CONFIG_RANDOM, CONFIG_GRID = 0, 1
    POSITION, VELOCITY = 0, 1

    def __init__(self, num_particles: int, grid_size=(64, 64, 64)):
        self.n = int(num_particles)
        self._h = lib.fcdemPS_create(self.n, *[int(g) for g in grid_size])
        if not self._h:
            raise MemoryError("fcdemPS_create failed")
        check("ParticleSystem()")

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib.fcdemPS_destroy(h)
            self._h = None

    @property
    def params(self) -> SimParams:
        return lib.fcdemPS_params(self._h).contents

    def update(self, dt: float) -> None:
        lib.fcdemPS_update(self._h, dt)

    def update_steps(self, dt: float, steps: int) -> None:
        lib.fcdemPS_updateSteps(self._h, dt, steps)

    def reset(self, config: int) -> None:
        lib.fcdemPS_reset(self._h, config)

    def set_array(self, array: int, data: np.ndarray, start: int = 0,
                  count: int | None = None) -> None:
        data = np.ascontiguousarray(data, np.float32)
        count = data.shape[0] if count is None else count
        lib.fcdemPS_setArray(self._h, array, data.ctypes.data, start, count)

    def get_array(self, array: int) -> np.ndarray:
        p = lib.fcdemPS_getArray(self._h, array)
        return np.ctypeslib.as_array(p, shape=(self.n, 4)).copy()

    def dump_grid(self) -> int:
        return int(lib.fcdemPS_dumpGrid(self._h))

    def set_fused_update(self, fused: bool) -> None:
        lib.fcdemPS_setFusedUpdate(self._h, int(fused))

    def set_radius_from_w(self, on: bool) -> None:
        lib.fcdemPS_setRadiusFromW(self._h, int(on))


# --- distance maps and the particledem_um entry points ----------------------

_DM_SIGS = {
    "fcdemDistMapCreate": (C.c_void_p, [C.c_void_p, C.c_void_p, C.POINTER(C.c_float),
                                        C.POINTER(C.c_float), C.c_float, C.POINTER(C.c_int)]),
    "fcdemDistMapTorus": (C.c_void_p, [C.c_float, C.c_float, C.c_int, C.c_float]),
    "fcdemDistMapDestroy": (None, [C.c_void_p]),
    "fcdemDistMapFromMesh": (C.c_void_p, [C.c_void_p, C.c_uint, C.c_void_p, C.c_uint, C.c_int,
                                          C.c_float]),
    "fcdemDistMapGeometry": (None, [C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_float),
                                    C.POINTER(C.c_float), C.POINTER(C.c_int)]),
    "fcdemDistMapVertices": (None, [C.c_void_p, C.c_void_p]),
    "fcdemDistMapQuery": (None, [C.c_void_p, C.c_void_p, C.c_uint, C.c_void_p, C.c_void_p]),
    "fcdemUM_integrateSystem": (None, [C.c_void_p, C.c_void_p, C.c_float, C.c_uint,
                                       C.c_void_p]),
    "fcdemUM_evalForces": (None, [C.c_void_p] * 7 + [C.c_uint, C.c_uint]),
    "fcdemUM_reorderDataAndFindCellStart": (None, [C.c_void_p] * 8 + [C.c_uint, C.c_uint]),
}
for _n, (_r, _a) in _DM_SIGS.items():
    getattr(lib, _n).restype = _r
    getattr(lib, _n).argtypes = _a


def _f3(v):
    return (C.c_float * 3)(*[float(x) for x in v])


class DistanceMap:
    """A distance map on the device (DistanceMap<float,gpu>,
    cuda_addon/distancemap.cuh:6-116)."""

    def __init__(self, handle):
        if not handle:
            raise MemoryError("distance map creation failed")
        self._h = handle
        vmin, vmax = (C.c_float * 3)(), (C.c_float * 3)()
        cs, cells = C.c_float(), (C.c_int * 3)()
        lib.fcdemDistMapGeometry(handle, vmin, vmax, C.byref(cs), cells)
        self.vmin, self.vmax = np.array(vmin, np.float32), np.array(vmax, np.float32)
        self.cell_size, self.cells = cs.value, np.array(cells, np.int32)

    @classmethod
    def from_arrays(cls, distance, contact_points, vmin, vmax, cell_size, cells):
        d = np.ascontiguousarray(distance, np.float32)
        c = np.ascontiguousarray(contact_points, np.float32)
        h = lib.fcdemDistMapCreate(d.ctypes.data, c.ctypes.data, _f3(vmin), _f3(vmax),
                                   float(cell_size), (C.c_int * 3)(*[int(x) for x in cells]))
        check("fcdemDistMapCreate")
        return cls(h)

    @classmethod
    def rounded_box(cls, half_extents, rounding=0.02, cells_per_axis=128, margin=0.05):
        h = lib.fcdemDistMapRoundedBox(_f3(half_extents), rounding, cells_per_axis, margin)
        check("fcdemDistMapRoundedBox")
        return cls(h)

    @classmethod
    def from_mesh(cls, vertices, triangles, cells_per_axis=128, margin=0.05):
        """Map of a closed, outward-oriented triangle mesh computed on the GPU
        (vertices (nv, 3) float, triangles (nt, 3) vertex indices)."""
        v = np.ascontiguousarray(vertices, np.float32)
        t = np.ascontiguousarray(triangles, np.uint32)
        h = lib.fcdemDistMapFromMesh(v.ctypes.data, v.shape[0], t.ctypes.data, t.shape[0],
                                     cells_per_axis, margin)
        check("fcdemDistMapFromMesh")
        return cls(h)

    @classmethod
    def torus(cls, major_radius=0.3, tube_radius=0.1, cells_per_axis=128, margin=0.05):
        h = lib.fcdemDistMapTorus(major_radius, tube_radius, cells_per_axis, margin)
        check("fcdemDistMapTorus")
        return cls(h)

    @property
    def handle(self):
        return self._h

    def vertices(self) -> np.ndarray:
        nv = int(np.prod(self.cells + 1))
        out = np.zeros((nv, 4), np.float32)
        lib.fcdemDistMapVertices(self._h, out.ctypes.data)
        check("fcdemDistMapVertices")
        return out

    def query(self, q: torch.Tensor):
        n = q.shape[0]
        dist = torch.empty(n, dtype=torch.float32, device=q.device)
        cp = torch.empty((n, 4), dtype=torch.float32, device=q.device)
        lib.fcdemDistMapQuery(self._h, _p(q), n, _p(dist), _p(cp))
        return dist, cp

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib.fcdemDistMapDestroy(h)
            self._h = None


def um_integrate_system(pos, vel, dt: float, n: int, dmap: DistanceMap | None) -> None:
    lib.fcdemUM_integrateSystem(_p(pos), _p(vel), dt, n, dmap.handle if dmap else None)


class RigidBody(C.Structure):
    """fcdemRigidBody: i3d::Rbody<float>'s fields (cuda_addon/rbody.hpp)."""
    _fields_ = [("numParticles", C.c_int), ("indices", C.c_int * 3), ("com", C.c_float * 3),
                ("vel", C.c_float * 3)]


lib.fcdemUM_integrateRigidBodies.argtypes = [C.c_void_p, C.c_uint, C.c_void_p, C.c_uint,
                                             C.c_float]
lib.fcdemUM_integrateRigidBodies.restype = None


def um_integrate_rigid_bodies(bodies: torch.Tensor, num_bodies: int, pos, n: int,
                              dt: float) -> None:
    """bodies: a device byte tensor holding num_bodies RigidBody records."""
    lib.fcdemUM_integrateRigidBodies(_p(bodies), num_bodies, _p(pos), n, dt)


def um_eval_forces(new_vel, force, sorted_pos, sorted_vel, index, cell_start, cell_end,
                   n: int, num_cells: int) -> None:
    lib.fcdemUM_evalForces(_p(new_vel), _p(force), _p(sorted_pos), _p(sorted_vel), _p(index),
                           _p(cell_start), _p(cell_end), n, num_cells)


def um_reorder(cell_start, cell_end, sorted_pos, sorted_vel, hash_, index, old_pos, old_vel,
               n: int, num_cells: int) -> None:
    lib.fcdemUM_reorderDataAndFindCellStart(_p(cell_start), _p(cell_end), _p(sorted_pos),
                                            _p(sorted_vel), _p(hash_), _p(index), _p(old_pos),
                                            _p(old_vel), n, num_cells)


lib.fcdemUM_update.argtypes = [C.c_void_p] * 9 + [C.c_float, C.c_uint, C.c_uint, C.c_uint,
                                                  C.c_void_p, C.c_void_p, C.c_float,
                                                  C.c_void_p]
lib.fcdemUM_update.restype = None


class UmScene(DeviceScene):
    """A scene on the unified-memory DEM path (particledem_um.cu): the
    ParticleWorld arrays plus force_, the distance-map obstacle, and the step
    of CollisionPipeline<dem_gpu_unified> (dempipeline.hpp:113-120)."""

    def __init__(self, scene: dict, dmap: DistanceMap | None = None,
                 device: str | torch.device = "cuda"):
        super().__init__(scene, device)
        self.dmap = dmap
        self.force = torch.zeros((self.n, 3), dtype=torch.float32, device=self.pos.device)

    def stages(self, dt: float | None = None) -> None:
        """One step as the reference issues it: calcHash, sortParticles,
        reorderDataAndFindCellStart, evalForces, integrateSystem."""
        dt = self.dt if dt is None else dt
        self.activate()
        calc_hash(self.hash, self.index, self.pos, self.n)
        sort_particles(self.hash, self.index, self.n)
        um_reorder(self.cell_start, self.cell_end, self.sorted_pos, self.sorted_vel, self.hash,
                   self.index, self.pos, self.vel, self.n, self.num_cells)
        um_eval_forces(self.vel, self.force, self.sorted_pos, self.sorted_vel, self.index,
                       self.cell_start, self.cell_end, self.n, self.num_cells)
        um_integrate_system(self.pos, self.vel, dt, self.n, self.dmap)

    def update(self, steps: int = 1, dt: float | None = None, net=None, skin: float = 0.0,
               exact_counter: torch.Tensor | None = None, force: bool = True) -> None:
        """`steps` steps through the fused fcdemUM_update; with `net` (an
        sdf.SdfNet) the map query is culled where the network predicts a
        distance above `skin`."""
        dt = self.dt if dt is None else dt
        self.activate()
        lib.fcdemUM_update(_p(self.pos), _p(self.vel), _p(self.force) if force else None,
                           _p(self.sorted_pos), _p(self.sorted_vel), _p(self.hash),
                           _p(self.index), _p(self.cell_start), _p(self.cell_end), dt, self.n,
                           self.num_cells, steps, self.dmap.handle if self.dmap else None,
                           net.handle if net is not None else None, skin,
                           _p(exact_counter) if exact_counter is not None else None)


# --- batches of scenes --------------------------------------------------------

class _BatchScene(C.Structure):
    _fields_ = [("params", SimParams), ("boxLo", C.c_float * 3), ("boxHi", C.c_float * 3),
                ("numParticles", C.c_uint)]


_B_SIGS = {
    "fcdemBatchCreate": (C.c_void_p, [C.POINTER(_BatchScene), C.c_uint, C.c_int]),
    "fcdemBatchDestroy": (None, [C.c_void_p]),
    "fcdemBatchNumParticles": (C.c_uint, [C.c_void_p]),
    "fcdemBatchNumCells": (C.c_uint, [C.c_void_p]),
    "fcdemBatchUpdate": (None, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_float, C.c_uint,
                                C.c_int]),
    "fcdemBatchSetObstacles": (None, [C.c_void_p, C.POINTER(C.c_void_p), C.c_uint,
                                      C.POINTER(C.c_int), C.c_void_p, C.c_float]),
    "fcdemBatchExactQueries": (C.c_ulonglong, [C.c_void_p, C.c_int]),
    "fcdemDistMapRoundedBox": (C.c_void_p, [C.POINTER(C.c_float), C.c_float, C.c_int,
                                            C.c_float]),
}
for _n, (_r, _a) in _B_SIGS.items():
    getattr(lib, _n).restype = _r
    getattr(lib, _n).argtypes = _a


class Batch:
    """Independent scenes stepped together (fcdemBatch*): scene dicts with
    pos, vel, params, box_lo, box_hi; their particles concatenated on the
    device in scene order."""

    def __init__(self, scene_list: list, device: str | torch.device = "cuda"):
        if not scene_list:
            raise ValueError("empty batch")
        w = {bool(s.get("radius_from_w", False)) for s in scene_list}
        if len(w) != 1:
            raise ValueError("all scenes of a batch share the radius mode")
        self.radius_from_w = w.pop()
        self.dt = float(scene_list[0].get("dt", 0.5))
        arr = (_BatchScene * len(scene_list))()
        for k, s in enumerate(scene_list):
            arr[k].params = s["params"]
            lo = s.get("box_lo", (-1.0, -1.0, -1.0))
            hi = s.get("box_hi", (1.0, 1.0, 1.0))
            arr[k].boxLo[:] = [float(x) for x in lo]
            arr[k].boxHi[:] = [float(x) for x in hi]
            arr[k].numParticles = int(s["pos"].shape[0])
        self._h = lib.fcdemBatchCreate(arr, len(scene_list), int(self.radius_from_w))
        check("fcdemBatchCreate")
        if not self._h:
            raise MemoryError("fcdemBatchCreate failed")
        self.sizes = [int(s["pos"].shape[0]) for s in scene_list]
        self.n = int(lib.fcdemBatchNumParticles(self._h))
        self.num_cells = int(lib.fcdemBatchNumCells(self._h))
        dev = torch.device(device)
        self.pos = torch.from_numpy(np.concatenate([s["pos"] for s in scene_list])).to(dev)
        self.vel = torch.from_numpy(np.concatenate([s["vel"] for s in scene_list])).to(dev)

    def update(self, steps: int = 1, dt: float | None = None, graph: bool = True) -> None:
        lib.fcdemBatchUpdate(self._h, _p(self.pos), _p(self.vel),
                             self.dt if dt is None else dt, steps, int(graph))

    def set_obstacles(self, maps: list, scene_shape, net=None, skin: float = 0.0) -> None:
        """Scene s gets obstacle maps[scene_shape[s]] (-1: none); with `net`
        (an sdf.SdfNet) the map query is culled above `skin`."""
        self._maps = list(maps)  # keep them alive while the batch uses them
        self._net = net
        hs = (C.c_void_p * max(len(maps), 1))(*[m.handle for m in maps])
        sh = (C.c_int * len(self.sizes))(*[int(x) for x in scene_shape])
        lib.fcdemBatchSetObstacles(self._h, hs, len(maps), sh,
                                   net.handle if net is not None else None, skin)
        check("fcdemBatchSetObstacles")

    def exact_queries(self, reset: bool = False) -> int:
        v = int(lib.fcdemBatchExactQueries(self._h, int(reset)))
        check("fcdemBatchExactQueries")
        return v

    def split(self, t: torch.Tensor) -> list:
        return list(torch.split(t, self.sizes))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib.fcdemBatchDestroy(h)
            self._h = None
