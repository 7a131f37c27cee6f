"""Seeded synthetic scenes (host numpy arrays) for the particle-DEM step.

Every scene is a dict with ``pos`` and ``vel`` ((n, 4) float32), ``params``
(SimParams), ``radius_from_w`` (polydisperse mode) and ``dt``.  The reference
ships no benchmark data: these generators restate its scene set-up
(particleSystem.cpp:380-402, particledem_um.cu:233-326) and extend it to the
polydisperse packed case.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from .params import SimParams, make_params

_f32p = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
_GEN = None


def _declare(lib):
    lib.fcdemSceneLattice.argtypes = [_f32p, _f32p, C.c_uint, C.c_float, C.c_float,
                                      C.c_float, C.c_float, C.c_ulonglong]
    lib.fcdemSceneLattice.restype = None
    lib.fcdemScenePack.argtypes = [_f32p, _f32p, C.c_uint, _f32p, _f32p, C.c_float,
                                   C.c_float, C.c_float, C.c_float, C.c_ulonglong, C.c_uint]
    lib.fcdemScenePack.restype = C.c_uint
    lib.fcdemScenePackRadii.argtypes = [_f32p, _f32p, C.c_uint, _f32p, _f32p, _f32p,
                                        C.c_float, C.c_ulonglong, C.c_uint]
    lib.fcdemScenePackRadii.restype = C.c_uint
    return lib


def use_generator(lib) -> None:
    """Builds scenes with the generator entry points of `lib` (a ctypes
    library exporting fcdemSceneLattice / fcdemScenePack /
    fcdemScenePackRadii) instead of libfcdem.so's."""
    global _GEN
    _GEN = _declare(lib)


def _lib():
    global _GEN
    if _GEN is None:
        from . import _native
        _GEN = _declare(_native.lib)
    return _GEN


def lattice(n: int, radius: float, jitter: float, vel_range: float, seed: int,
            spacing: float | None = None):
    pos = np.zeros((n, 4), np.float32)
    vel = np.zeros((n, 4), np.float32)
    sp = 2.0 * radius if spacing is None else spacing
    _lib().fcdemSceneLattice(pos, vel, n, radius, sp, jitter, vel_range, seed)
    return pos, vel


def pack(n: int, box_min, box_max, r_median: float, sigma: float, r_max: float,
         vel_range: float, seed: int, max_attempts: int = 20000):
    pos = np.zeros((n, 4), np.float32)
    vel = np.zeros((n, 4), np.float32)
    placed = _lib().fcdemScenePack(pos, vel, n, np.asarray(box_min, np.float32),
                                 np.asarray(box_max, np.float32), r_median, sigma,
                                 r_max, vel_range, seed, max_attempts)
    if placed != n:
        raise RuntimeError(f"packing placed {placed} of {n} spheres")
    return pos, vel


def lattice_scene(n: int = 16384, seed: int = 1973) -> dict:
    """Plain DEM: n monodisperse spheres of radius 1/64 on a jittered lattice
    (spacing 2r, jitter 0.01r) in the [-1,1]^3 box, 64^3 grid with cell = 2r,
    velocities U[-0.01, 0.01], gravity -3e-4, spring 0.5, damping 0.02,
    shear 0.1, attraction 0, boundary damping -0.5, dt 0.5."""
    r = 1.0 / 64.0
    pos, vel = lattice(n, r, 0.01 * r, 0.01, seed)
    return dict(name="plain-16k-64^3", pos=pos, vel=vel,
                params=make_params(n, (64, 64, 64), r), radius_from_w=False, dt=0.5)


def lognormal_mean_volume(r_median: float, sigma: float) -> float:
    return 4.0 / 3.0 * math.pi * r_median ** 3 * math.exp(4.5 * sigma * sigma)


def packed_scene(n: int = 4194304, seed: int = 2024, grid: int = 256,
            volume_fraction: float = 0.30) -> dict:
    """Plain DEM at scale: n spheres with lognormal radii (median 1/512,
    sigma 0.25, clipped at 2/512), cell = max diameter (grid cells span the
    [-1,1] box), random sequential packing at the given volume fraction in a
    centred cube, the contact parameters of lattice_scene.  Smaller n keep the
    radii and the packing density (the cube shrinks)."""
    r_med, sigma, r_max = 1.0 / 512.0, 0.25, 2.0 / 512.0
    vol = n * lognormal_mean_volume(r_med, sigma)
    side = (vol / volume_fraction) ** (1.0 / 3.0)
    side = min(side, 2.0 - 4.0 * r_max)
    lo = [-side / 2.0] * 3
    hi = [side / 2.0] * 3
    pos, vel = pack(n, lo, hi, r_med, sigma, r_max, 0.01, seed)
    cell = 2.0 * r_max
    g = grid
    p = make_params(n, (g, g, g), particle_radius=r_max, cell_size=cell)
    return dict(name=f"packed-{n}-{g}^3", pos=pos, vel=vel, params=p,
                radius_from_w=True, dt=0.5, box_side=side)


def torus_fall_scene(n: int = 1048576, seed: int = 2, grid: int = 256, z0: float = 0.15) -> dict:
    """Spheres falling onto a torus (the distance-map obstacle): n spheres of
    radius 1/256 on a jittered lattice (spacing 2.2 r, jitter 0.05 r),
    128 x 128 columns wide, centred over the torus (R 0.3, r 0.1, in the
    z = 0 plane) and starting at z = z0; velocities U[-0.001, 0.001];
    gravity -3e-4 along z, the contact parameters of lattice_scene, dt 0.5; grid^3
    cells of one diameter from (-1, -1, -1); no collider sphere (the
    unified-memory evalForces has none)."""
    r = 1.0 / 256.0
    sp = 2.2 * r
    nx = ny = 128 if n >= 128 * 128 else max(1, int(np.sqrt(n)))
    nz = (n + nx * ny - 1) // (nx * ny)
    rng = np.random.default_rng(seed)
    k = np.arange(n)
    ix, iy, iz = k % nx, (k // nx) % ny, k // (nx * ny)
    pos = np.zeros((n, 4), np.float32)
    pos[:, 0] = (ix - (nx - 1) / 2.0) * sp
    pos[:, 1] = (iy - (ny - 1) / 2.0) * sp
    pos[:, 2] = z0 + iz * sp
    pos[:, :3] += rng.uniform(-0.05 * r, 0.05 * r, (n, 3))
    pos[:, 3] = 1.0
    vel = np.zeros((n, 4), np.float32)
    vel[:, :3] = rng.uniform(-0.001, 0.001, (n, 3))
    p = make_params(n, (grid, grid, grid), r, gravity=(0.0, 0.0, -3e-4),
                    collider_pos=(10.0, 10.0, 10.0), collider_radius=0.0)
    return dict(name=f"torus-{n}", pos=pos, vel=vel, params=p, radius_from_w=False, dt=0.5,
                radius=r)


def random_box(n: int, grid=(16, 16, 16), radius: float = 1.0 / 16.0, seed: int = 7,
               vel_range: float = 0.01, cell: float | None = None,
               origin=(-1.0, -1.0, -1.0), poly: bool = False) -> dict:
    """Uniform random positions in [-1,1]^3 (overlaps allowed), as
    ParticleSystem::reset(CONFIG_RANDOM) places them."""
    rng = np.random.default_rng(seed)
    pos = np.zeros((n, 4), np.float32)
    pos[:, :3] = rng.uniform(-1.0, 1.0, (n, 3)).astype(np.float32)
    if poly:
        pos[:, 3] = rng.uniform(0.5 * radius, radius, n).astype(np.float32)
    else:
        pos[:, 3] = 1.0
    vel = np.zeros((n, 4), np.float32)
    vel[:, :3] = rng.uniform(-vel_range, vel_range, (n, 3)).astype(np.float32)
    p = make_params(n, grid, radius, cell_size=cell, world_origin=origin)
    return dict(name=f"random-{n}", pos=pos, vel=vel, params=p, radius_from_w=poly,
                dt=0.5)


def pack_radii(radii: np.ndarray, box_min, box_max, vel_range: float, seed: int,
               max_attempts: int = 20000):
    n = radii.shape[0]
    pos = np.zeros((n, 4), np.float32)
    vel = np.zeros((n, 4), np.float32)
    placed = _lib().fcdemScenePackRadii(pos, vel, n, np.ascontiguousarray(radii, np.float32),
                                      np.asarray(box_min, np.float32),
                                      np.asarray(box_max, np.float32), vel_range, seed,
                                      max_attempts)
    if placed != n:
        raise RuntimeError(f"packing placed {placed} of {n} spheres")
    return pos, vel


def _pow2_at_least(x: int) -> int:
    g = 1
    while g < x:
        g *= 2
    return g


def batch_scene(n: int, seed: int, volume_fraction: float = 0.25, r_min: float = 1.0 / 512.0,
                r_max: float = 1.0 / 256.0) -> dict:
    """One scene of the batched workload: n spheres with radii U[r_min, r_max]
    packed at the volume fraction in a cube of side L centred at the origin,
    which is also the scene's box; grid cells of 2 r_max, the grid the next
    power of two of cells covering the box."""
    rng = np.random.default_rng(seed)
    radii = rng.uniform(r_min, r_max, n).astype(np.float32)
    vol = float((4.0 / 3.0 * np.pi * radii.astype(np.float64) ** 3).sum())
    side = (vol / volume_fraction) ** (1.0 / 3.0)
    lo, hi = [-side / 2.0] * 3, [side / 2.0] * 3
    pos, vel = pack_radii(radii, lo, hi, 0.01, seed + 1)
    cell = 2.0 * r_max
    g = max(4, _pow2_at_least(int(np.ceil(side / cell))))
    p = make_params(n, (g, g, g), particle_radius=r_max, cell_size=cell,
                    world_origin=(-side / 2.0,) * 3, collider_pos=(10.0, 10.0, 10.0),
                    collider_radius=0.0)
    return dict(name=f"batch-scene-{n}", pos=pos, vel=vel, params=p, radius_from_w=True,
                dt=0.5, box_lo=np.array(lo, np.float32), box_hi=np.array(hi, np.float32))


def batch_box_scenes(num_scenes: int = 512, n_min: int = 1024, n_max: int = 65536,
                  seed: int = 3) -> list:
    """Batched plain DEM: scene sizes drawn log-uniform in [n_min, n_max]
    (seeded), radii U[1/512, 1/256], 25% volume fraction per scene."""
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(n_min), np.log(n_max), num_scenes)).astype(np.int64)
    return [batch_scene(int(n), seed * 100003 + k) for k, n in enumerate(sizes)]


def obstacle_set(num: int = 8, seed: int = 41) -> list:
    """The procedural obstacles of the batched neural-SDF workload: half tori
    (major radius U[0.2, 0.35], tube radius U[0.05, 0.12]) and half rounded
    boxes (half-extents U[0.1, 0.3] per axis, rounding 0.02), seeded; each a
    dict kind/params, centred at the origin."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(num):
        if k % 2 == 0:
            out.append(dict(kind="torus", R=float(rng.uniform(0.2, 0.35)),
                            r=float(rng.uniform(0.05, 0.12))))
        else:
            out.append(dict(kind="box", h=[float(x) for x in rng.uniform(0.1, 0.3, 3)],
                            rounding=0.02))
    return out


def obstacle_top(ob: dict) -> float:
    return ob["r"] if ob["kind"] == "torus" else ob["h"][2]


def obstacle_scene(n: int, ob: dict, seed: int, r_min: float = 1.0 / 512.0,
                   r_max: float = 1.0 / 256.0) -> dict:
    """One scene of the batched neural-SDF workload: n spheres with radii
    U[r_min, r_max] on a jittered lattice (spacing 2.05 r_max, at most
    120 x 120 columns) starting one diameter above the obstacle's top,
    falling (gravity -3e-4 along z) onto it inside the box [-0.5, 0.5]^3;
    128^3 grid cells of one max diameter; the contact parameters of lattice_scene."""
    rng = np.random.default_rng(seed)
    sp = 2.05 * r_max
    nx = ny = min(120, max(1, int(np.ceil(np.sqrt(n)))))
    k = np.arange(n)
    ix, iy, iz = k % nx, (k // nx) % ny, k // (nx * ny)
    pos = np.zeros((n, 4), np.float32)
    pos[:, 0] = (ix - (nx - 1) / 2.0) * sp
    pos[:, 1] = (iy - (ny - 1) / 2.0) * sp
    pos[:, 2] = obstacle_top(ob) + 2.0 * r_max + iz * sp
    pos[:, :3] += rng.uniform(-0.02 * r_max, 0.02 * r_max, (n, 3))
    pos[:, 3] = rng.uniform(r_min, r_max, n)
    vel = np.zeros((n, 4), np.float32)
    vel[:, :3] = rng.uniform(-0.001, 0.001, (n, 3))
    p = make_params(n, (128, 128, 128), particle_radius=r_max, cell_size=2.0 * r_max,
                    world_origin=(-0.5, -0.5, -0.5), gravity=(0.0, 0.0, -3e-4),
                    collider_pos=(10.0, 10.0, 10.0), collider_radius=0.0)
    return dict(name=f"obstacle-scene-{n}", pos=pos, vel=vel, params=p, radius_from_w=True,
                dt=0.5, box_lo=np.array([-0.5] * 3, np.float32),
                box_hi=np.array([0.5] * 3, np.float32))


def batch_obstacle_scenes(num_scenes: int = 128, n_min: int = 4096, n_max: int = 262144,
                  seed: int = 4, num_shapes: int = 8):
    """Batched DEM with obstacles: scene sizes log-uniform in [n_min, n_max]
    (seeded), scene s over obstacle s % num_shapes.  Returns (scenes,
    obstacles, scene_shape)."""
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(n_min), np.log(n_max), num_scenes)).astype(np.int64)
    obs = obstacle_set(num_shapes)
    shape = [k % num_shapes for k in range(num_scenes)]
    scs = [obstacle_scene(int(n), obs[shape[k]], seed * 100003 + k) for k, n in enumerate(sizes)]
    return scs, obs, shape


def torus_mesh(major_radius: float = 0.3, tube_radius: float = 0.1, nu: int = 256,
               nv: int = 64):
    """The procedural torus obstacle as a closed triangle mesh: nu x nv quads
    of the (u around z, v around the tube) parametrisation
    ((R + r cos v) cos u, (R + r cos v) sin u, r sin v), each split into two
    triangles ordered so that their normals point outwards.  Returns
    (vertices (nu*nv, 3) float32, triangles (2*nu*nv, 3) uint32)."""
    u = 2.0 * np.pi * np.arange(nu) / nu
    v = 2.0 * np.pi * np.arange(nv) / nv
    U, V = np.meshgrid(u, v, indexing="ij")
    rho = major_radius + tube_radius * np.cos(V)
    verts = np.stack([rho * np.cos(U), rho * np.sin(U), tube_radius * np.sin(V)], -1)
    verts = verts.reshape(-1, 3).astype(np.float32)
    i, j = np.meshgrid(np.arange(nu), np.arange(nv), indexing="ij")
    a = i * nv + j
    b = ((i + 1) % nu) * nv + j
    c = ((i + 1) % nu) * nv + (j + 1) % nv
    d = i * nv + (j + 1) % nv
    tris = np.concatenate([np.stack([a, b, c], -1).reshape(-1, 3),
                           np.stack([a, c, d], -1).reshape(-1, 3)]).astype(np.uint32)
    return verts, tris
