"""Distance-map row on the GPU: the query and the particledem_um boundary
integrate against the reference's own code (golden fixture), the torus map
generator against the analytic torus, and the particledem_um evalForces /
reorder variants against the oracle."""
import numpy as np
import pytest
import torch

from fcdem_testutil import GOLDEN, REL_TOL, force_floor, oracle_params, rel_err_vec

pytestmark = pytest.mark.gpu


def _fixture():
    with np.load(f"{GOLDEN}/distmap_torus.npz") as z:
        return {k: z[k] for k in z.files}


def _map(g):
    from fullc0ntact_gb300 import dem
    return dem.DistanceMap.from_arrays(g["distance"], g["contact_points"], g["vmin"], g["vmax"],
                                       float(g["cell_size"]), g["cells"])


def test_query_matches_reference_fixture():
    g = _fixture()
    m = _map(g)
    q = np.zeros((g["queries"].shape[0], 4), np.float32)
    q[:, :3] = g["queries"]
    dist, cp = m.query(torch.from_numpy(q).cuda())
    dist, cp = dist.cpu().numpy(), cp.cpu().numpy()[:, :3]
    # the distance interpolation runs in double as in the reference: bit-exact
    np.testing.assert_array_equal(dist.view(np.uint32), g["dist"].view(np.uint32))
    inside = g["dist"] != 5.0
    # contact points: float FMA contraction may move the last bit
    err = np.abs(cp[inside] - g["cp"][inside]).max()
    assert err <= 2e-7, err


def test_um_integrate_matches_reference_fixture():
    from fullc0ntact_gb300 import dem
    from fullc0ntact_gb300.params import make_params
    g = _fixture()
    m = _map(g)
    P = make_params(g["pos0"].shape[0], (4, 4, 4), float(g["radius"]),
                    gravity=tuple(g["gravity"]), global_damping=float(g["global_damping"]),
                    boundary_damping=float(g["boundary_damping"]))
    dem.set_parameters(P)
    dem.set_radius_mode(False)
    pos = torch.from_numpy(g["pos0"].copy()).cuda()
    vel = torch.from_numpy(g["vel0"].copy()).cuda()
    dem.um_integrate_system(pos, vel, float(g["dt"]), pos.shape[0], m)
    dem.check("fcdemUM_integrateSystem")
    p, v = pos.cpu().numpy(), vel.cpu().numpy()
    # The push direction normalize(pos - cp) is ill-conditioned for particles
    # within ~1e-4 of the surface: last-bit differences of the interpolated
    # contact point (FMA contraction here, none in the host build) and of
    # rsqrtf (hardware) grow by 1/|pos - cp|.  Positions: 1e-5 of the unit
    # domain (the push itself is >= 0.1 r = 1.6e-3); velocities: 1e-5 relative.
    assert np.abs(p[:, :3] - g["pos"][:, :3]).max() <= 1e-5
    assert rel_err_vec(v, g["vel"], 1e-6).max() <= REL_TOL
    np.testing.assert_array_equal(p[:, 3], g["pos"][:, 3])
    np.testing.assert_array_equal(v[:, 3], g["pos"][:, 3])  # vel.w = pos.w


def test_torus_generator_matches_analytic_torus():
    from fullc0ntact_gb300 import dem
    from oracle import oracle as O
    m = dem.DistanceMap.torus(0.3, 0.1, 64, 0.05)
    v = m.vertices()
    coords = O.lattice_coords(m.vmin, m.cell_size, m.cells).astype(np.float64)
    rho = np.hypot(coords[:, 0], coords[:, 1])
    sd = np.sqrt((rho - 0.3) ** 2 + coords[:, 2] ** 2) - 0.1
    assert np.abs(v[:, 0] - sd).max() <= 1e-6
    # contact points lie on the torus surface
    cp = v[:, 1:].astype(np.float64)
    on = np.sqrt((np.hypot(cp[:, 0], cp[:, 1]) - 0.3) ** 2 + cp[:, 2] ** 2) - 0.1
    assert np.abs(on).max() <= 1e-6
    # a query at a vertex returns its distance
    q = np.zeros((1, 4), np.float32)
    q[0, :3] = coords[1234]
    d, _ = m.query(torch.from_numpy(q).cuda())
    assert abs(float(d.cpu()[0]) - v[1234, 0]) <= 1e-6


def test_um_eval_forces_and_reorder_match_oracle():
    from fullc0ntact_gb300 import dem, scenes
    from oracle import oracle as O
    sc = scenes.random_box(8000, grid=(32, 32, 32), radius=1.0 / 40.0, seed=21)
    ds = dem.DeviceScene(sc)
    ds.activate()
    n, nc = ds.n, ds.num_cells
    dem.calc_hash(ds.hash, ds.index, ds.pos, n)
    dem.sort_particles(ds.hash, ds.index, n)
    dem.um_reorder(ds.cell_start, ds.cell_end, ds.sorted_pos, ds.sorted_vel, ds.hash, ds.index,
                   ds.pos, ds.vel, n, nc)
    force = torch.zeros((n, 3), dtype=torch.float32, device="cuda")
    nv = torch.zeros_like(ds.vel)
    dem.um_eval_forces(nv, force, ds.sorted_pos, ds.sorted_vel, ds.index, ds.cell_start,
                       ds.cell_end, n, nc)
    dem.check("particledem_um")
    ce = ds.cell_end.cpu().numpy().view(np.uint32)
    cs = ds.cell_start.cpu().numpy().view(np.uint32)
    assert np.all(ce[cs == 0xFFFFFFFF] == 0xFFFFFFFF)  # cellEnd reset as well
    P = oracle_params(bytes(sc["params"]))
    h, x = O.calc_hash(P, sc["pos"])
    hs, xs = O.sort_pairs(h, x)
    ocs, oce, sp, sv = O.reorder(hs, xs, sc["pos"], sc["vel"], P.numCells)
    onv, of = O.collide(P, sp, sv, xs, ocs, oce, with_collider=False, want_force=True)
    f = force.cpu().numpy()
    assert rel_err_vec(f, of, force_floor(of)).max() <= REL_TOL
    assert rel_err_vec(nv.cpu().numpy(), onv, 1e-6).max() <= REL_TOL
