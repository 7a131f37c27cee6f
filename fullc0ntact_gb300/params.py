"""The SimParams block (cuda_addon/particles_kernel.cuh:27-48) and the
parameter sets of the reference's scenes."""
from __future__ import annotations

import ctypes as C


class SimParams(C.Structure):
    """104 bytes, 4-byte aligned; field order and offsets of the reference."""

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

    def copy(self) -> "SimParams":
        return SimParams.from_buffer_copy(bytes(self))


assert C.sizeof(SimParams) == 104

OFFSETS = {name: getattr(SimParams, name).offset for name, _ in SimParams._fields_}


def make_params(num_bodies: int, grid=(64, 64, 64), particle_radius: float = 1.0 / 64.0,
                cell_size: float | None = None, world_origin=(-1.0, -1.0, -1.0),
                spring=0.5, damping=0.02, shear=0.1, attraction=0.0,
                boundary_damping=-0.5, gravity=(0.0, 0.0, -0.0003), global_damping=1.0,
                collider_pos=(-1.2, -0.8, 0.8), collider_radius=0.2) -> SimParams:
    """Parameters as ParticleSystem's constructor sets them
    (particleSystem.cpp:30-72): cell size = particle diameter unless given,
    origin (-1,-1,-1), collider sphere at (-1.2,-0.8,0.8) with radius 0.2."""
    p = SimParams()
    p.colliderPos[:] = list(collider_pos)
    p.colliderRadius = collider_radius
    p.gravity[:] = list(gravity)
    p.globalDamping = global_damping
    p.particleRadius = particle_radius
    p.gridSize[:] = list(grid)
    p.numCells = grid[0] * grid[1] * grid[2]
    p.worldOrigin[:] = list(world_origin)
    cs = 2.0 * particle_radius if cell_size is None else cell_size
    p.cellSize[:] = [cs, cs, cs]
    p.numBodies = num_bodies
    p.maxParticlesPerCell = 0
    p.spring = spring
    p.damping = damping
    p.shear = shear
    p.attraction = attraction
    p.boundaryDamping = boundary_damping
    return p
