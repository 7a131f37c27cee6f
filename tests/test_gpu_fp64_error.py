"""The FP32 force error against an FP64 evaluation of the same collide (the
oracle's FP64 twin on the same sorted arrays), stated per workload: the
packed polydisperse scene, the torus-fall scene's evalForces (force_
output, no collider), a scene with collapsed cells (the crowded-
neighbourhood kernel), the largest kind of scene of the batched workload
(65,536 spheres, radii U[1/512, 1/256], 25% packing) and a scene of the
batched obstacle workload after 150 batched steps onto its rounded box (a
batch gives each scene the bits of that scene alone).  The error is
relative to max(|F|, median |F|)."""
import numpy as np
import pytest

from fcdem_testutil import force_floor, rel_err_vec

pytestmark = pytest.mark.gpu


def _collapsed(sc, counts, cells):
    rng = np.random.default_rng(9)
    cell = float(sc["params"].cellSize[0])
    origin = np.array([sc["params"].worldOrigin[k] for k in range(3)], np.float32)
    picks = rng.permutation(sc["pos"].shape[0])
    s = 0
    for cnt, c in zip(counts, cells):
        idx = picks[s:s + cnt]
        s += cnt
        lo = origin + np.array(c, np.float32) * cell
        sc["pos"][idx, :3] = lo + rng.uniform(0.05, 0.95, (cnt, 3)).astype(np.float32) * cell
    return sc


def _obstacle_pile(steps=150):
    """A batched-obstacle scene after `steps` batched steps onto its obstacle
    (the first rounded box of the obstacle set)."""
    from fullc0ntact_gb300 import dem, scenes, sdf
    obs = scenes.obstacle_set()
    ob = next(o for o in obs if o["kind"] != "torus")
    sc = scenes.obstacle_scene(120_000, ob, seed=7)
    b = dem.Batch([sc])
    b.set_obstacles(sdf.obstacle_maps([ob], 64), [0])
    b.update(steps, graph=False)
    dem.check("obstacle batch")
    return dict(sc, pos=b.pos.cpu().numpy().copy(), vel=b.vel.cpu().numpy().copy())


@pytest.mark.parametrize("kind", ["packed", "collapsed", "torus_um", "batch_scene",
                                  "obstacle_pile"])
def test_force_error_against_fp64(kind):
    from fullc0ntact_gb300 import dem, scenes
    from oracle import oracle as O
    if kind == "packed":
        sc = scenes.packed_scene(200_000, grid=128)
    elif kind == "batch_scene":
        sc = scenes.batch_scene(65_536, seed=17)
    elif kind == "obstacle_pile":
        sc = _obstacle_pile()
    elif kind == "collapsed":
        sc = _collapsed(scenes.packed_scene(100_000, grid=128), (2500, 700, 300),
                        ((5, 5, 5), (6, 5, 5), (9, 9, 9)))
    else:
        sc = scenes.torus_fall_scene(200_000, z0=0.095)
    P = O.SimParams.from_buffer_copy(bytes(sc["params"]))
    w = bool(sc.get("radius_from_w", False))
    if kind == "torus_um":
        # 60 steps onto the torus first: the lattice starts without contacts
        dmap = dem.DistanceMap.torus(0.3, 0.1, 128, 0.05)
        ds = dem.UmScene(sc, dmap)
        ds.update(60)
        sc = dict(sc, vel=ds.vel.cpu().numpy().copy())
        ds.activate()
        dem.calc_hash(ds.hash, ds.index, ds.pos, ds.n)
        dem.sort_particles(ds.hash, ds.index, ds.n)
        dem.um_reorder(ds.cell_start, ds.cell_end, ds.sorted_pos, ds.sorted_vel, ds.hash,
                       ds.index, ds.pos, ds.vel, ds.n, ds.num_cells)
        dem.um_eval_forces(ds.vel, ds.force, ds.sorted_pos, ds.sorted_vel, ds.index,
                           ds.cell_start, ds.cell_end, ds.n, ds.num_cells)
        dem.check("um")
        f32 = ds.force.cpu().numpy().astype(np.float64)
        nv64 = O.collide_f64(P, ds.sorted_pos.cpu().numpy(), ds.sorted_vel.cpu().numpy(),
                             dem.u32(ds.index), dem.u32(ds.cell_start), dem.u32(ds.cell_end),
                             radius_from_w=w, with_collider=False)
        f64 = nv64[:, :3] - sc["vel"][:, :3].astype(np.float64)
    else:
        ds = dem.DeviceScene(sc)
        ds.stages()
        dem.check("stages")
        st = O.step_stages(P, sc["pos"], sc["vel"], sc["dt"], radius_from_w=w)
        nv64 = O.collide_f64(P, st["sortedPos"], st["sortedVel"], st["index_sorted"],
                             st["cellStart"], st["cellEnd"], radius_from_w=w)
        f64 = nv64[:, :3] - st["vel_in"][:, :3].astype(np.float64)
        f32 = ds.vel.cpu().numpy()[:, :3].astype(np.float64) - st["vel_in"][:, :3]
    assert int((np.abs(f64).sum(axis=1) > 0).sum()) > 1000  # contacts to judge
    err = rel_err_vec(f32, f64, force_floor(f64))
    print(f"{kind}: force error vs FP64 max {err.max():.3e} median {np.median(err):.3e} "
          f"p99.9 {np.quantile(err, 0.999):.3e}")
    assert err.max() < 1e-3
    assert np.quantile(err, 0.999) < 1e-5
