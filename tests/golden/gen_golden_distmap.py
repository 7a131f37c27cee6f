"""Golden fixtures of the distance-map row from the reference's OWN code:
cuda_addon/distancemap.cuh (queryMap) and cuda_addon/boundaries.cuh
(d_checkBoundaryDistMap), built as host code (oracle/_ref/libfcref_distmap.so,
recipe in oracle/Makefile).  Run where the reference tree is present:
    make -C oracle all ref && python tests/golden/gen_golden_distmap.py

The map is the torus around z with R = 0.3, r = 0.1 (the obstacle of the
benchmark set), sampled exactly at the vertices of a 24 x 24 x 8-cell lattice
(closest point and signed distance of the analytic torus, in float64 and
stored as float32).  Fixture keys: vmin, vmax, cell_size, cells, distance,
contact_points (the reference's host layout), queries/dist/cp (queryMap),
and an integrate case: pos0/vel0 -> pos/vel with params gravity, damping,
dt, radius, boundary damping.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import oracle as O  # noqa: E402


def torus_map(R=0.3, r=0.1, cells_xy=24, margin=0.05):
    ex = R + r + margin
    cs = np.float32(2.0 * ex / cells_xy)
    cz = int(np.ceil(2.0 * (r + margin) / cs))
    vmin = np.array([-ex, -ex, -0.5 * cz * cs], np.float32)
    cells = np.array([cells_xy, cells_xy, cz], np.int32)
    vmax = (vmin + cells.astype(np.float32) * cs).astype(np.float32)
    coords = O.lattice_coords(vmin, cs, cells)
    p = coords.astype(np.float64)
    rho = np.hypot(p[:, 0], p[:, 1])
    q = np.stack([R * p[:, 0] / rho, R * p[:, 1] / rho, np.zeros_like(rho)], 1)
    d = p - q
    dq = np.linalg.norm(d, axis=1)
    cp = q + r * d / dq[:, None]
    dist = (dq - r).astype(np.float32)
    return dict(vmin=vmin, vmax=vmax, cell_size=cs, cells=cells, distance=dist,
                contact_points=np.ascontiguousarray(cp.astype(np.float32)), coords=coords)


def main():
    L = O.ref_distmap()
    if L is None:
        raise SystemExit("oracle/_ref/libfcref_distmap.so missing: run `make -C oracle all ref`")
    rng = np.random.default_rng(77)
    m = torus_map()
    n = 4000
    # queries inside the box (away from the upper faces), plus outside points
    span = m["vmax"] - m["vmin"]
    qi = m["vmin"] + rng.uniform(0.0, 0.999, (n, 3)).astype(np.float32) * span
    qo = rng.uniform(-1.0, 1.0, (200, 3)).astype(np.float32)
    q = np.ascontiguousarray(np.concatenate([qi, qo]).astype(np.float32))
    dist = np.zeros(q.shape[0], np.float32)
    cp = np.zeros_like(q)
    L.fcref_distmap_query(m["distance"], m["contact_points"], m["coords"], m["vmin"], m["vmax"],
                          float(m["cell_size"]), m["cells"], q, q.shape[0], dist, cp)
    # particles falling onto the torus: positions near its surface
    k = 3000
    pos0 = np.zeros((k, 4), np.float32)
    ang = rng.uniform(0, 2 * np.pi, k)
    phi = rng.uniform(0, 2 * np.pi, k)
    rr = 0.1 + rng.uniform(-0.01, 0.02, k)
    pos0[:, 0] = (0.3 + rr * np.cos(phi)) * np.cos(ang)
    pos0[:, 1] = (0.3 + rr * np.cos(phi)) * np.sin(ang)
    pos0[:, 2] = rr * np.sin(phi)
    pos0[:, 3] = 1.0
    pos0[:50, :2] *= 4.0  # some outside the r = 1 cylinder
    vel0 = np.zeros((k, 4), np.float32)
    vel0[:, :3] = rng.uniform(-0.01, 0.01, (k, 3))
    grav = np.array([0.0, 0.0, -3e-4], np.float32)
    pos, vel = pos0.copy(), vel0.copy()
    normals = np.zeros_like(m["contact_points"])
    L.fcref_um_integrate(m["distance"], m["contact_points"], m["coords"], normals, m["vmin"],
                         m["vmax"], float(m["cell_size"]), m["cells"], pos, vel, k, grav, 1.0,
                         0.5, 1.0 / 64.0, -0.5)
    path = os.path.join(HERE, "distmap_torus.npz")
    np.savez_compressed(path, vmin=m["vmin"], vmax=m["vmax"], cell_size=m["cell_size"],
                        cells=m["cells"], distance=m["distance"],
                        contact_points=m["contact_points"], queries=q, dist=dist, cp=cp,
                        pos0=pos0, vel0=vel0, pos=pos, vel=vel, gravity=grav,
                        global_damping=np.float32(1.0), dt=np.float32(0.5),
                        radius=np.float32(1.0 / 64.0), boundary_damping=np.float32(-0.5))
    print(path, os.path.getsize(path), "bytes;", int((dist < 1.0 / 64.0).sum()),
          "queries within one radius")


if __name__ == "__main__":
    main()
