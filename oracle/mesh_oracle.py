"""FP64 CPU oracle of the triangle-mesh distance map.

Test infrastructure only: the tests import it to check the GPU generator
(fcdemDistMapFromMesh).  At a query point: the distance to the closest point
of the mesh over all triangles (the closest point of a triangle taken from
the plane projection or, outside the triangle, the closest point of its
edges), negative when the generalized winding number (summed signed solid
angles over 4 pi, Van Oosterom and Strackee 1983) exceeds 1/2; and that
closest point -- what DistanceMapMesh::ComputeDistance
(inshape3dcore/distance/distancegridcgal.hpp:36-69) stores per vertex.
"""
from __future__ import annotations

import numpy as np


def _closest_on_segment(p, a, b):
    ab = b - a
    t = np.clip(np.einsum("...k,...k", p - a, ab) / np.maximum(np.einsum("...k,...k", ab, ab), 1e-300), 0.0, 1.0)
    return a + t[..., None] * ab


def closest_on_triangles(p, A, B, C):
    """Closest points of triangles (A, B, C) (each (nt, 3)) to points p (np, 3):
    (np, nt, 3)."""
    p = p[:, None, :]
    n = np.cross(B - A, C - A)
    nn = np.einsum("tk,tk->t", n, n)
    t = np.einsum("ptk,tk->pt", p - A[None], n) / nn
    q = p - t[..., None] * n[None]
    # barycentric inside test of the projection
    c0 = np.einsum("ptk,tk->pt", np.cross(B - A, q - A[None]), n)
    c1 = np.einsum("ptk,tk->pt", np.cross(C - B, q - B[None]), n)
    c2 = np.einsum("ptk,tk->pt", np.cross(A - C, q - C[None]), n)
    inside = (c0 >= 0) & (c1 >= 0) & (c2 >= 0)
    e0 = _closest_on_segment(p, A[None], B[None])
    e1 = _closest_on_segment(p, B[None], C[None])
    e2 = _closest_on_segment(p, C[None], A[None])
    cands = np.stack([e0, e1, e2], 0)
    d = np.linalg.norm(cands - p[None], axis=-1)
    best = np.take_along_axis(cands, np.argmin(d, 0)[None, ..., None], 0)[0]
    return np.where(inside[..., None], q, best)


def winding_number(p, A, B, C):
    a = A[None] - p[:, None]
    b = B[None] - p[:, None]
    c = C[None] - p[:, None]
    la, lb, lc = (np.linalg.norm(x, axis=-1) for x in (a, b, c))
    det = np.einsum("ptk,ptk->pt", a, np.cross(b, c))
    den = (la * lb * lc + np.einsum("ptk,ptk->pt", a, b) * lc +
           np.einsum("ptk,ptk->pt", a, c) * lb + np.einsum("ptk,ptk->pt", b, c) * la)
    return (2.0 * np.arctan2(det, den)).sum(1) / (4.0 * np.pi)


def mesh_distance(points, vertices, triangles, chunk=256):
    """(signed distance (np,), closest point (np, 3)) in FP64."""
    V = np.asarray(vertices, np.float64)
    T = np.asarray(triangles, np.int64)
    A, B, C = V[T[:, 0]], V[T[:, 1]], V[T[:, 2]]
    P = np.asarray(points, np.float64)
    dist = np.empty(len(P))
    cp = np.empty((len(P), 3))
    for s in range(0, len(P), chunk):
        p = P[s:s + chunk]
        q = closest_on_triangles(p, A, B, C)
        d = np.linalg.norm(q - p[:, None], axis=-1)
        k = np.argmin(d, 1)
        dmin = d[np.arange(len(p)), k]
        w = winding_number(p, A, B, C)
        dist[s:s + chunk] = np.where(w > 0.5, -dmin, dmin)
        cp[s:s + chunk] = q[np.arange(len(p)), k]
    return dist, cp
