"""The oracle's batched-scene restatements (CPU only):

* the box integrate in the reference's [-1,1]^3 box is the reference's
  integrate (the oracle's restatement, and the reference's own code built
  as host code where present), bit for bit at the workloads' dt = 0.5;
* the obstacle integrate without a map is the box integrate;
* its map contact agrees with the restatement of checkDistMap
  (boundaries.cuh:38-63), pinned to the reference fixture, within the
  roundings of the fused multiply-adds: velocities bit for bit, positions
  within 1e-5 (the contact normal normalises p - cp, and near the surface
  one rounding of the contact point turns its direction), and it pushes the touching
  spheres that touch it from outside away from it."""
import numpy as np
import pytest

from fcdem_testutil import GOLDEN
from oracle import oracle as O


def _scene(n=4000, seed=3):
    rng = np.random.default_rng(seed)
    pos = np.zeros((n, 4), np.float32)
    pos[:, :3] = rng.uniform(-1.05, 1.05, (n, 3))
    pos[:, 3] = rng.uniform(1 / 512, 1 / 256, n)
    vel = np.zeros((n, 4), np.float32)
    vel[:, :3] = rng.uniform(-0.02, 0.02, (n, 3))
    P = O.SimParams()
    P.gravity[:] = [0.0, 0.0, -3e-4]
    P.globalDamping = 1.0
    P.particleRadius = 1 / 256
    P.boundaryDamping = -0.5
    return P, pos, vel


def test_box_integrate_in_reference_box_is_reference_integrate():
    P, pos, vel = _scene()
    a, av = pos.copy(), vel.copy()
    b, bv = pos.copy(), vel.copy()
    O.integrate(P, a, av, 0.5, True)
    O.integrate_box(P, [-1, -1, -1], [1, 1, 1], b, bv, 0.5, True)
    np.testing.assert_array_equal(a.view(np.uint32), b.view(np.uint32))
    np.testing.assert_array_equal(av.view(np.uint32), bv.view(np.uint32))
    L = O.ref_host()
    if L is not None:  # the reference's own integrate_functor, monodisperse
        c, cv = pos.copy(), vel.copy()
        d, dv = pos.copy(), vel.copy()
        L.fcref_setParameters(P)
        L.fcref_integrateSystem(c, cv, 0.5, c.shape[0])
        O.integrate_box(P, [-1, -1, -1], [1, 1, 1], d, dv, 0.5, False)
        np.testing.assert_array_equal(c.view(np.uint32), d.view(np.uint32))
        np.testing.assert_array_equal(cv.view(np.uint32), dv.view(np.uint32))


def test_box_integrate_clamps_to_its_box():
    P, pos, vel = _scene(seed=4)
    lo, hi = np.array([-0.3, -0.2, -0.1], np.float32), np.array([0.3, 0.25, 0.4], np.float32)
    O.integrate_box(P, lo, hi, pos, vel, 0.5, True)
    r = pos[:, 3:4]
    assert np.all(pos[:, :3] >= lo + r) and np.all(pos[:, :3] <= hi - r)


def test_obstacle_integrate_without_map_is_box_integrate():
    P, pos, vel = _scene(seed=5)
    lo, hi = [-0.5] * 3, [0.5] * 3
    a, av = pos.copy(), vel.copy()
    b, bv = pos.copy(), vel.copy()
    O.integrate_box(P, lo, hi, a, av, 0.5, True)
    assert O.batch_obstacle_integrate(P, lo, hi, None, b, bv, 0.5, True) == 0
    np.testing.assert_array_equal(a.view(np.uint32), b.view(np.uint32))
    np.testing.assert_array_equal(av.view(np.uint32), bv.view(np.uint32))


def test_obstacle_contact_agrees_with_check_distmap():
    with np.load(f"{GOLDEN}/distmap_torus.npz") as z:
        g = {k: z[k] for k in z.files}
    m = O.distmap_struct(g["vmin"], g["vmax"], float(g["cell_size"]), g["cells"],
                         np.ascontiguousarray(g["distance"]),
                         np.ascontiguousarray(g["contact_points"]))
    rng = np.random.default_rng(8)
    n = 6000
    r = np.float32(1 / 256)
    # points near the torus surface (R 0.3, r 0.1 in the z = 0 plane)
    u, v = rng.uniform(0, 2 * np.pi, n), rng.uniform(0, 2 * np.pi, n)
    rho = rng.uniform(0.1 - 2 * r, 0.1 + 3 * r, n)
    pos = np.zeros((n, 4), np.float32)
    pos[:, 0] = (0.3 + rho * np.cos(v)) * np.cos(u)
    pos[:, 1] = (0.3 + rho * np.cos(v)) * np.sin(u)
    pos[:, 2] = rho * np.sin(v)
    pos[:, 3] = r
    vel = np.zeros((n, 4), np.float32)
    P = O.SimParams()
    P.globalDamping = 1.0
    P.particleRadius = r
    P.boundaryDamping = -0.5
    a, av = pos.copy(), vel.copy()
    nc = O.batch_obstacle_integrate(P, [-1] * 3, [1] * 3, m, a, av, 0.5, False)
    assert nc > 1000
    b, bv = pos.copy(), vel.copy()
    lib = O.lib()
    import ctypes as C
    for i in range(n):
        p3, v3 = b[i, :3].copy(), bv[i, :3].copy()
        lib.orc_check_distmap(C.byref(m), C.c_float(r), C.c_float(-0.5),
                              p3.ctypes.data_as(C.POINTER(C.c_float)),
                              v3.ctypes.data_as(C.POINTER(C.c_float)))
        b[i, :3], bv[i, :3] = p3, v3
    np.testing.assert_allclose(a[:, :3], b[:, :3], rtol=0, atol=1e-5)
    np.testing.assert_array_equal(av.view(np.uint32), bv.view(np.uint32))
    moved = np.any(a[:, :3] != pos[:, :3], axis=1)
    assert moved.sum() == nc
    # a sphere touching from outside (0 < d < r) moves away from the surface
    out = [i for i in np.flatnonzero(moved)[:800] if O.distmap_query(m, pos[i, :3])[0] > 0]
    d0 = np.array([O.distmap_query(m, pos[i, :3])[0] for i in out])
    d1 = np.array([O.distmap_query(m, a[i, :3])[0] for i in out])
    assert len(out) > 100 and np.mean(d1 > d0) > 0.99  # the map is coarse (cell 9.6 r)
