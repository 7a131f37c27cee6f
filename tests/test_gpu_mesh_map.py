"""The GPU triangle-mesh distance map (fcdemDistMapFromMesh): at every vertex
of a coarse torus mesh's map, the FP64 oracle's signed distance and closest
point; the config-2 mesh (256 x 64 quads) on the 128-cell map agrees with the
exact torus map within the faceting error."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_mesh_map_matches_fp64_oracle():
    from fullc0ntact_gb300 import dem, scenes
    from oracle import mesh_oracle as mo
    from oracle import oracle as O
    verts, tris = scenes.torus_mesh(0.3, 0.1, 24, 10)
    m = dem.DistanceMap.from_mesh(verts, tris, 24, 0.05)
    v = m.vertices()
    coords = O.lattice_coords(m.vmin, m.cell_size, m.cells).astype(np.float64)
    d, cp = mo.mesh_distance(coords, verts, tris)
    assert np.abs(v[:, 0] - d).max() <= 2e-6
    assert np.all(np.sign(v[np.abs(d) > 1e-5, 0]) == np.sign(d[np.abs(d) > 1e-5]))
    # the contact point is a closest point: |vertex - cp| = |distance|
    gcp = v[:, 1:].astype(np.float64)
    assert np.abs(np.linalg.norm(coords - gcp, axis=1) - np.abs(d)).max() <= 2e-6
    # and lies on the mesh (where several triangles are equally close -- the
    # symmetry planes of the lattice -- it may be another one than the
    # oracle's)
    on, _ = mo.mesh_distance(gcp, verts, tris)
    assert np.abs(on).max() <= 2e-6


def test_torus_mesh_map_matches_exact_torus():
    from fullc0ntact_gb300 import dem, scenes
    R, r = 0.3, 0.1
    verts, tris = scenes.torus_mesh(R, r, 256, 64)
    m = dem.DistanceMap.from_mesh(verts, tris, 128, 0.05)
    t = dem.DistanceMap.torus(R, r, 128, 0.05)
    assert np.allclose(m.vmin, t.vmin, atol=1e-6) and np.allclose(m.vmax, t.vmax, atol=1e-6)
    vm, vt = m.vertices(), t.vertices()
    facet = r * (1 - np.cos(np.pi / 64)) + (R + r) * (1 - np.cos(np.pi / 256))
    assert np.abs(vm[:, 0] - vt[:, 0]).max() <= facet + 1e-5
    far = np.abs(vt[:, 0]) > 2 * facet
    assert np.all(np.sign(vm[far, 0]) == np.sign(vt[far, 0]))
