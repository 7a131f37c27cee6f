"""Generates the golden fixtures of tests/golden/ from the reference's OWN
kernel code: cuda_addon/particles_kernel.cu built as host code
(oracle/_ref/libfcref_host.so, recipe in oracle/Makefile), driven with the
launch glue of cuda_addon/particleSystem.cu.

Run it where the reference tree is present:
    make -C oracle all ref && python tests/golden/gen_golden.py

Each fixture holds the inputs of one ParticleSystem::update and the output of
every stage as the reference computes it:
    params (104 raw bytes), dt, pos0/vel0 (inputs), pos/vel (after
    integrateSystem), hash/index (calcHash), hash_sorted/index_sorted
    (sortParticles), cells/cell_start/cell_end (non-empty cells only),
    new_vel (collide).
sortedPos/sortedVel are pos[index_sorted]/vel[index_sorted] and not stored.
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402


def params_block(grid, radius, cell=None, origin=(-1.0, -1.0, -1.0), n=0,
                 collider=(-1.2, -0.8, 0.8), collider_r=0.2, attraction=0.0):
    p = O.SimParams()
    p.colliderPos[:] = list(collider)
    p.colliderRadius = collider_r
    p.gravity[:] = [0.0, 0.0, -0.0003]
    p.globalDamping = 1.0
    p.particleRadius = radius
    p.gridSize[:] = list(grid)
    p.numCells = grid[0] * grid[1] * grid[2]
    p.worldOrigin[:] = list(origin)
    c = 2.0 * radius if cell is None else cell
    p.cellSize[:] = [c, c, c]
    p.numBodies = n
    p.spring, p.damping, p.shear, p.attraction, p.boundaryDamping = 0.5, 0.02, 0.1, attraction, -0.5
    return p


def lattice(n, radius, jitter, vel_range, rng):
    side = int(np.ceil(n ** (1.0 / 3.0) - 1e-9))
    while side ** 3 < n:
        side += 1
    idx = np.arange(n)
    x, y, z = idx % side, (idx // side) % side, idx // (side * side)
    pos = np.zeros((n, 4), np.float32)
    sp = np.float32(2.0 * radius)
    for k, c in enumerate((x, y, z)):
        pos[:, k] = (sp * c.astype(np.float32) + np.float32(radius) - np.float32(1.0)
                     + (rng.uniform(-1, 1, n) * jitter).astype(np.float32))
    pos[:, 3] = 1.0
    vel = np.zeros((n, 4), np.float32)
    vel[:, :3] = rng.uniform(-vel_range, vel_range, (n, 3)).astype(np.float32)
    return pos, vel


def run_reference(P, pos0, vel0, dt):
    R = O.ref_host()
    n = pos0.shape[0]
    pos, vel = pos0.copy(), vel0.copy()
    R.fcref_setParameters(C.byref(P))
    R.fcref_integrateSystem(pos, vel, dt, n)
    h = np.empty(n, np.uint32)
    x = np.empty(n, np.uint32)
    R.fcref_calcHash(h, x, pos, n)
    hs, xs = h.copy(), x.copy()
    R.fcref_sortParticles(hs, xs, n)
    cs = np.empty(P.numCells, np.uint32)
    ce = np.full(P.numCells, 0xFFFFFFFF, np.uint32)
    sp, sv = np.empty_like(pos), np.empty_like(vel)
    R.fcref_reorderDataAndFindCellStart(cs, ce, sp, sv, hs, xs, pos, vel, n, P.numCells)
    nv = vel.copy()
    R.fcref_collide(nv, sp, sv, xs, cs, ce, n, P.numCells)
    cells = np.nonzero(cs != 0xFFFFFFFF)[0].astype(np.uint32)
    return dict(pos=pos, vel=vel, hash=h, index=x, hash_sorted=hs, index_sorted=xs,
                cells=cells, cell_start=cs[cells], cell_end=ce[cells], new_vel=nv)


def cases():
    rng = np.random.default_rng(20241203)
    out = {}
    # the lattice scene: 16384 spheres r = 1/64 on the jittered
    # lattice, 64^3 grid.
    r = 1.0 / 64.0
    pos, vel = lattice(16384, r, 0.01 * r, 0.01, rng)
    out["plain16k"] = (params_block((64, 64, 64), r, n=16384), pos, vel, 0.5)
    # random positions (overlaps, collider contacts), 16^3 grid, r = 1/16 as
    # ParticleSystem's defaults; n not a multiple of any block size.
    n = 3001
    pos = np.zeros((n, 4), np.float32)
    pos[:, :3] = rng.uniform(-1.0, 1.0, (n, 3)).astype(np.float32)
    pos[:, 3] = 1.0
    vel = np.zeros((n, 4), np.float32)
    vel[:, :3] = rng.uniform(-0.05, 0.05, (n, 3)).astype(np.float32)
    out["random3001"] = (params_block((16, 16, 16), 1.0 / 16.0, n=n), pos, vel, 0.5)
    # wrap-around: a 4^3 grid over a box smaller than the particle domain, so
    # hashes alias and the 27 neighbour cells wrap; attraction on.
    n = 700
    pos = np.zeros((n, 4), np.float32)
    pos[:, :3] = rng.uniform(-1.0, 1.0, (n, 3)).astype(np.float32)
    pos[:, 3] = 1.0
    vel = np.zeros((n, 4), np.float32)
    vel[:, :3] = rng.uniform(-0.02, 0.02, (n, 3)).astype(np.float32)
    out["wrap700"] = (params_block((4, 4, 4), 0.08, cell=0.25, n=n, attraction=0.01),
                      pos, vel, 0.25)
    # particles exactly on cell faces (x, y, z multiples of the cell size)
    n = 512
    g = rng.integers(0, 32, (n, 3))
    pos = np.zeros((n, 4), np.float32)
    pos[:, :3] = (g.astype(np.float32) * np.float32(1.0 / 16.0) - np.float32(1.0))
    pos[:, 3] = 1.0
    vel = np.zeros((n, 4), np.float32)
    out["faces512"] = (params_block((32, 32, 32), 1.0 / 32.0, n=n), pos, vel, 0.0)
    # everything in one cell
    n = 40
    pos = np.zeros((n, 4), np.float32)
    pos[:, :3] = rng.uniform(0.01, 0.05, (n, 3)).astype(np.float32)
    pos[:, 3] = 1.0
    vel = np.zeros((n, 4), np.float32)
    vel[:, :3] = rng.uniform(-0.01, 0.01, (n, 3)).astype(np.float32)
    out["onecell40"] = (params_block((8, 8, 8), 0.125, cell=0.25, n=n), pos, vel, 0.1)
    # a single particle touching the collider sphere
    pos = np.array([[-0.95, -0.75, 0.7, 1.0]], np.float32)
    vel = np.array([[0.001, -0.002, 0.003, 0.0]], np.float32)
    out["single1"] = (params_block((16, 16, 16), 1.0 / 16.0, n=1), pos, vel, 0.5)
    return out


def main():
    if not O.ref_host_available():
        raise SystemExit("oracle/_ref/libfcref_host.so is missing: run `make -C oracle all ref` "
                         "where the reference tree is present")
    for name, (P, pos0, vel0, dt) in cases().items():
        res = run_reference(P, pos0, vel0, dt)
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(path, params=np.frombuffer(bytes(P), np.uint8), dt=np.float32(dt),
                            pos0=pos0, vel0=vel0, **res)
        print(f"{path}: n={pos0.shape[0]} cells={res['cells'].size} "
              f"size={os.path.getsize(path)} B")


if __name__ == "__main__":
    main()
