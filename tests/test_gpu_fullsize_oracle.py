"""Single-step parity with the oracle at the full sizes of the two large
single-scene workloads, on the same input state:

* the packed polydisperse scene, 4,194,304 spheres in a 256^3 grid, at
  three points of its 500-step job: the packed start, step 200 (settled
  layers, crowded neighbourhoods) and step 450 (tens of thousands of
  particles with NaN coordinates in a few cells).  One fcdemUpdate call
  against one oracle update (integrate, calcHash, sort, reorder, collide)
  with the GPU's fused arithmetic: every output bit for bit.  The error of
  the oracle's host arithmetic (every product rounded) against the GPU is
  printed: in the settled states a few particles sum many large pair terms
  to a small net force, and the two roundings disagree there by more than
  the net force's 1e-5;
* a 100,000-sphere version of the packed scene, 100 steps: the trajectory
  ends in the oracle's bits;
* the torus fall, 1,048,576 spheres of radius 1/256 onto the 128-cell
  distance map built from the 256 x 64-quad torus mesh, after 60 steps (the
  spheres on the torus).  One fused unified-memory step (fcdemUM_update:
  calcHash, sort, reorder, evalForces, the integrate with the map, cylinder
  and planes) against the oracle's composition of the same calls (fused
  arithmetic): sorted arrays and evalForces' force bit for bit, velocities
  bit for bit, positions within 2e-7 (the GPU normalises the contact normal
  with rsqrtf, within 2 ulp of the oracle's 1/sqrtf); and the same step with
  the neural SDF culling the map query ends in the same bits."""
import numpy as np
import pytest
import torch

from fcdem_testutil import (REL_TOL, assert_same_floats, check_cell_tables, force_floor,
                            oracle_params, rel_err_vec)

pytestmark = pytest.mark.gpu


def _bits(t):
    return t.view(torch.int32)


def test_packed_full_size_single_steps_match_oracle():
    from fullc0ntact_gb300 import dem, scenes
    from oracle import oracle as O
    sc = scenes.packed_scene(4_194_304)
    P = oracle_params(bytes(sc["params"]))
    ds = dem.DeviceScene(sc)
    done = 0
    for at in (0, 200, 450):
        if at > done:
            ds.update(at - done)
            dem.check("advance")
            done = at
        pos, vel = ds.pos.cpu().numpy().copy(), ds.vel.cpu().numpy().copy()
        ds.update(1)
        dem.check("update")
        done += 1
        with O.gpu_arithmetic():
            st = O.step_stages(P, pos, vel, sc["dt"], radius_from_w=True)
        assert_same_floats(ds.pos.cpu().numpy(), st["pos"])
        np.testing.assert_array_equal(dem.u32(ds.hash), st["hash_sorted"])
        np.testing.assert_array_equal(dem.u32(ds.index), st["index_sorted"])
        check_cell_tables(dem.u32(ds.cell_start), dem.u32(ds.cell_end), st["cellStart"],
                          st["cellEnd"])
        assert_same_floats(ds.sorted_pos.cpu().numpy(), st["sortedPos"])
        assert_same_floats(ds.sorted_vel.cpu().numpy(), st["sortedVel"])
        assert_same_floats(ds.vel.cpu().numpy()[:, :3], st["newVel"][:, :3])
        # the host arithmetic on the same sorted input, for the record
        host = O.collide(P, st["sortedPos"], st["sortedVel"], st["index_sorted"],
                         st["cellStart"], st["cellEnd"], True, True)
        f_ref = host[:, :3].astype(np.float64) - st["vel_in"][:, :3]
        f_gpu = ds.vel.cpu().numpy()[:, :3].astype(np.float64) - st["vel_in"][:, :3]
        err = rel_err_vec(f_gpu, f_ref, force_floor(f_ref))
        nan = int(np.isnan(pos[:, :3]).any(axis=1).sum())
        print(f"step {at}: bit-exact; host arithmetic force error max {err.max():.2e}, "
              f"{int((err > REL_TOL).sum())} particles above 1e-5, {nan} NaN particles")


def test_packed_trajectory_ends_in_oracle_bits():
    from fullc0ntact_gb300 import dem, scenes
    from oracle import oracle as O
    sc = scenes.packed_scene(100_000, grid=128)
    P = oracle_params(bytes(sc["params"]))
    ds = dem.DeviceScene(sc)
    ds.update(100)
    dem.check("update")
    pos, vel = sc["pos"].copy(), sc["vel"].copy()
    with O.gpu_arithmetic():
        O.update(P, pos, vel, sc["dt"], steps=100, radius_from_w=True)
    assert_same_floats(ds.pos.cpu().numpy(), pos)
    assert_same_floats(ds.vel.cpu().numpy()[:, :3], vel[:, :3])


def _oracle_map(dmap):
    from oracle import oracle as O
    v = dmap.vertices()
    return O.distmap_struct(dmap.vmin, dmap.vmax, dmap.cell_size, dmap.cells,
                            np.ascontiguousarray(v[:, 0]), np.ascontiguousarray(v[:, 1:]))


def test_torus_fall_full_size_step_matches_oracle():
    from fullc0ntact_gb300 import dem, scenes, sdf
    from oracle import oracle as O
    sc = scenes.torus_fall_scene(1_048_576)
    verts, tris = scenes.torus_mesh(0.3, 0.1, 256, 64)
    dmap = dem.DistanceMap.from_mesh(verts, tris, 128, 0.05)
    ds = dem.UmScene(sc, dmap)
    ds.update(60)
    dem.check("advance")
    pos, vel = ds.pos.cpu().numpy().copy(), ds.vel.cpu().numpy().copy()
    ds.update(1)
    dem.check("um step")
    P = oracle_params(bytes(sc["params"]))
    w = bool(sc.get("radius_from_w", False))
    h, x = O.calc_hash(P, pos)
    hs, xs = O.sort_pairs(h, x)
    cs, ce, sp, sv = O.reorder(hs, xs, pos, vel, P.numCells)
    with O.gpu_arithmetic():
        nv, force = O.collide(P, sp, sv, xs, cs, ce, w, False, want_force=True)
    np.testing.assert_array_equal(dem.u32(ds.hash), hs)
    np.testing.assert_array_equal(dem.u32(ds.index), xs)
    check_cell_tables(dem.u32(ds.cell_start), dem.u32(ds.cell_end), cs, ce)
    assert_same_floats(ds.sorted_pos.cpu().numpy(), sp)
    assert_same_floats(ds.sorted_vel.cpu().numpy(), sv)
    assert_same_floats(ds.force.cpu().numpy(), force)
    po, vo = pos.copy(), nv.copy()
    m = _oracle_map(dmap)
    with O.gpu_arithmetic():
        O.integrate_distmap(P, m, po, vo, sc["dt"], w)
    pg, vg = ds.pos.cpu().numpy(), ds.vel.cpu().numpy()
    np.testing.assert_allclose(pg[:, :3], po[:, :3], rtol=0, atol=2e-7)
    assert_same_floats(vg[:, :3], vo[:, :3])
    # the host arithmetic, for the record
    _, host = O.collide(P, sp, sv, xs, cs, ce, w, False, want_force=True)
    ferr = rel_err_vec(ds.force.cpu().numpy(), host, force_floor(host))
    in_box = ((pos[:, :3] >= dmap.vmin) & (pos[:, :3] <= dmap.vmax)).all(axis=1)
    print(f"torus fall: bit-exact force and velocity, max position difference "
          f"{np.abs(pg[:, :3] - po[:, :3]).max():.2e}; host arithmetic force error "
          f"{ferr.max():.2e}; {int(in_box.sum())} spheres in the map box")
    # the same step with the network culling the map query: the same bits
    net = sdf.SdfNet(3, 64, 3, seed=5)
    net.normalize_to(dmap)
    train = sdf.samples(dmap, 2_000_000, 0.6, 0.05, seed=21)
    net.train(train, epochs=20, batch=2048, lr=5e-3, band=0.02)
    del train
    exact_pos, exact_vel = ds.pos.clone(), ds.vel.clone()
    ds.pos.copy_(torch.from_numpy(pos))
    ds.vel.copy_(torch.from_numpy(vel))
    counter = torch.zeros(1, dtype=torch.int32, device=ds.pos.device)
    ds.update(1, net=net, skin=2.0 * sc["radius"], exact_counter=counter)
    dem.check("um step, neural")
    assert torch.equal(_bits(ds.pos), _bits(exact_pos))
    assert torch.equal(_bits(ds.vel), _bits(exact_vel))
    print(f"neural: {int(counter.item())} exact map queries of {int(in_box.sum())} in the box")
