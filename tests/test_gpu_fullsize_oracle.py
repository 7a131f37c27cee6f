"""Single-step parity with the oracle at the full sizes of the two large
single-scene workloads, on the same input state:

* the packed polydisperse scene, 4,194,304 spheres in a 256^3 grid, at
  three points of its 500-step job: the packed start, step 200 (settled
  layers, crowded neighbourhoods) and step 450 (tens of thousands of
  particles with NaN coordinates in a few cells).  One fcdemUpdate call
  against one oracle update (integrate, calcHash, sort, reorder, collide):
  integrated positions, hashes, permutation, cell ranges and sorted arrays
  bit for bit, forces within 1e-5 of max(|F|, median |F|);
* the torus fall, 1,048,576 spheres of radius 1/256 onto the 128-cell
  distance map built from the 256 x 64-quad torus mesh, after 60 steps (the
  spheres on the torus).  One fused unified-memory step (fcdemUM_update:
  calcHash, sort, reorder, evalForces, the integrate with the map, cylinder
  and planes) against the oracle's composition of the same calls: sorted
  arrays bit for bit, evalForces' force within 1e-5, positions within 1e-7
  (the GPU normalises the contact normal with rsqrtf), velocities within
  1e-5 of the force scale; and the same step with the neural SDF culling
  the map query ends in the same bits."""
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
        st = O.step_stages(P, pos, vel, sc["dt"], radius_from_w=True)
        assert_same_floats(ds.pos.cpu().numpy(), st["pos"])
        np.testing.assert_array_equal(dem.u32(ds.hash), st["hash_sorted"])
        np.testing.assert_array_equal(dem.u32(ds.index), st["index_sorted"])
        check_cell_tables(dem.u32(ds.cell_start), dem.u32(ds.cell_end), st["cellStart"],
                          st["cellEnd"])
        assert_same_floats(ds.sorted_pos.cpu().numpy(), st["sortedPos"])
        assert_same_floats(ds.sorted_vel.cpu().numpy(), st["sortedVel"])
        f_ref = st["newVel"][:, :3].astype(np.float64) - st["vel_in"][:, :3]
        f_gpu = ds.vel.cpu().numpy()[:, :3].astype(np.float64) - st["vel_in"][:, :3]
        err = rel_err_vec(f_gpu, f_ref, force_floor(f_ref))
        nan = int(np.isnan(pos[:, :3]).any(axis=1).sum())
        print(f"step {at}: max force error {err.max():.2e} (median {np.median(err):.1e}), "
              f"{nan} NaN particles")
        assert err.max() <= REL_TOL, at


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
    nv, force = O.collide(P, sp, sv, xs, cs, ce, w, False, want_force=True)
    np.testing.assert_array_equal(dem.u32(ds.hash), hs)
    np.testing.assert_array_equal(dem.u32(ds.index), xs)
    check_cell_tables(dem.u32(ds.cell_start), dem.u32(ds.cell_end), cs, ce)
    assert_same_floats(ds.sorted_pos.cpu().numpy(), sp)
    assert_same_floats(ds.sorted_vel.cpu().numpy(), sv)
    floor = force_floor(force)
    ferr = rel_err_vec(ds.force.cpu().numpy(), force, floor)
    assert ferr.max() <= REL_TOL, float(ferr.max())
    po, vo = pos.copy(), nv.copy()
    m = _oracle_map(dmap)
    O.integrate_distmap(P, m, po, vo, sc["dt"], w)
    pg, vg = ds.pos.cpu().numpy(), ds.vel.cpu().numpy()
    np.testing.assert_allclose(pg[:, :3], po[:, :3], rtol=0, atol=1e-7)
    verr = np.linalg.norm(vg[:, :3].astype(np.float64) - vo[:, :3], axis=1) / floor
    assert verr.max() <= REL_TOL, float(verr.max())
    # map contacts in this step (the integrate changes these velocities)
    in_box = ((pos[:, :3] >= dmap.vmin) & (pos[:, :3] <= dmap.vmax)).all(axis=1)
    print(f"torus fall: force error {ferr.max():.2e}, velocity error {verr.max():.2e}, "
          f"{int(in_box.sum())} spheres in the map box")
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
