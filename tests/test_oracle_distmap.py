"""The oracle's distance-map query and boundary response against the
reference's own code (cuda_addon/distancemap.cuh, boundaries.cuh) via the
golden fixture, bit for bit."""
import numpy as np
import pytest

from fcdem_testutil import GOLDEN
from oracle import oracle as O


def _fixture():
    with np.load(f"{GOLDEN}/distmap_torus.npz") as z:
        return {k: z[k] for k in z.files}


def _oracle_map(g):
    return O.distmap_struct(g["vmin"], g["vmax"], float(g["cell_size"]), g["cells"],
                            np.ascontiguousarray(g["distance"]),
                            np.ascontiguousarray(g["contact_points"]))


def test_oracle_query_matches_reference_fixture():
    g = _fixture()
    m = _oracle_map(g)
    q = g["queries"]
    for i in range(q.shape[0]):
        d, cp = O.distmap_query(m, q[i])
        assert np.float32(d).view(np.uint32) == g["dist"][i].view(np.uint32), i
        if g["dist"][i] != 5.0:
            np.testing.assert_array_equal(cp.view(np.uint32), g["cp"][i].view(np.uint32))


def test_oracle_boundary_matches_reference_fixture():
    g = _fixture()
    m = _oracle_map(g)
    P = O.SimParams()
    P.gravity[:] = list(g["gravity"])
    P.globalDamping = float(g["global_damping"])
    P.particleRadius = float(g["radius"])
    P.boundaryDamping = float(g["boundary_damping"])
    pos, vel = g["pos0"].copy(), g["vel0"].copy()
    O.integrate_distmap(P, m, pos, vel, float(g["dt"]))
    np.testing.assert_array_equal(pos.view(np.uint32), g["pos"].view(np.uint32))
    np.testing.assert_array_equal(vel.view(np.uint32), g["vel"].view(np.uint32))
    moved = np.any(g["pos"][:, :3] != g["pos0"][:, :3] + 0.5 * g["vel0"][:, :3], axis=1)
    assert moved.sum() > 100  # the map and the cylinder push particles


@pytest.mark.skipif(O.ref_distmap() is None, reason="reference distance-map build absent")
def test_oracle_query_matches_reference_code_random_map():
    L = O.ref_distmap()
    rng = np.random.default_rng(5)
    cells = np.array([7, 5, 9], np.int32)
    cs = np.float32(0.0371)
    vmin = np.array([-0.2, 0.1, -0.05], np.float32)
    vmax = (vmin + cells.astype(np.float32) * cs).astype(np.float32)
    nv = int(np.prod(cells + 1))
    dist = rng.normal(0, 0.1, nv).astype(np.float32)
    cps = rng.normal(0, 0.3, (nv, 3)).astype(np.float32)
    coords = O.lattice_coords(vmin, cs, cells)
    q = (vmin + rng.uniform(0, 0.995, (2000, 3)).astype(np.float32) * (vmax - vmin)).astype(np.float32)
    rd = np.zeros(2000, np.float32)
    rcp = np.zeros((2000, 3), np.float32)
    L.fcref_distmap_query(dist, cps, coords, vmin, vmax, float(cs), cells,
                          np.ascontiguousarray(q), 2000, rd, rcp)
    m = O.distmap_struct(vmin, vmax, float(cs), cells, dist, cps)
    for i in range(2000):
        d, cp = O.distmap_query(m, q[i])
        assert np.float32(d) == rd[i]
        np.testing.assert_array_equal(cp, rcp[i])
