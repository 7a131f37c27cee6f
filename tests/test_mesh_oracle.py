"""The FP64 mesh-distance oracle against the exact torus: a fine torus mesh's
distance differs from the analytic torus distance by at most the faceting
error, and inside points get negative distances."""
import numpy as np

from fullc0ntact_gb300 import scenes
from oracle import mesh_oracle as mo


def test_mesh_oracle_matches_analytic_torus():
    R, r = 0.3, 0.1
    verts, tris = scenes.torus_mesh(R, r, 96, 32)
    rng = np.random.default_rng(1)
    p = rng.uniform([-0.5, -0.5, -0.2], [0.5, 0.5, 0.2], (400, 3))
    d, cp = mo.mesh_distance(p, verts, tris)
    exact = np.sqrt((np.hypot(p[:, 0], p[:, 1]) - R) ** 2 + p[:, 2] ** 2) - r
    facet = r * (1 - np.cos(np.pi / 32)) + (R + r) * (1 - np.cos(np.pi / 96)) + 1e-6
    assert np.abs(d - exact).max() <= facet
    assert np.all(np.sign(d[np.abs(exact) > 2 * facet]) == np.sign(exact[np.abs(exact) > 2 * facet]))
    # closest points lie on the mesh: |p - cp| = |d|
    assert np.abs(np.linalg.norm(p - cp, axis=1) - np.abs(d)).max() < 1e-12
