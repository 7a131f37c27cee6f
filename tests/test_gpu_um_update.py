"""The fused unified-memory step (fcdemUM_update: counting-sort pipeline,
evalForces, integrate with the distance-map boundary and the next hash)
leaves the same state as the reference-named staged calls; with the neural
SDF culling the map query it leaves the same state again."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _state(ds):
    start = ds.cell_start.cpu().numpy().view(np.uint32)
    end = ds.cell_end.cpu().numpy().view(np.uint32).copy()
    end[start == 0xFFFFFFFF] = 0xFFFFFFFF  # cellEnd of empty cells is not compared
    return dict(pos=ds.pos.cpu().numpy(), vel=ds.vel.cpu().numpy(),
                force=ds.force.cpu().numpy(), hash=ds.hash.cpu().numpy(),
                index=ds.index.cpu().numpy(), sorted_pos=ds.sorted_pos.cpu().numpy(),
                sorted_vel=ds.sorted_vel.cpu().numpy(), cell_start=start, cell_end=end)


def _same(a, b):
    for k in a:
        np.testing.assert_array_equal(np.asarray(a[k]).view(np.uint32),
                                      np.asarray(b[k]).view(np.uint32), err_msg=k)


@pytest.mark.parametrize("steps", [1, 4])
@pytest.mark.parametrize("with_map", [True, False])
def test_um_update_equals_staged(steps, with_map):
    from fullc0ntact_gb300 import dem, scenes
    dmap = dem.DistanceMap.torus(0.3, 0.1, 128, 0.05) if with_map else None
    # the lowest layers start in and just above the torus: the map pushes
    sc = scenes.torus_fall_scene(60_000, z0=0.09)
    a, b = dem.UmScene(sc, dmap), dem.UmScene(sc, dmap)
    for _ in range(steps):
        a.stages()
    b.update(steps)
    dem.check("um update")
    _same(_state(a), _state(b))


def test_um_update_with_sdf_culling_equals_exact_map():
    from fullc0ntact_gb300 import dem, scenes, sdf
    dmap = dem.DistanceMap.torus(0.3, 0.1, 128, 0.05)
    net = sdf.SdfNet(3, 64, 3, seed=5)
    net.normalize_to(dmap)
    net.train(sdf.samples(dmap, 2_000_000, 0.6, 0.05, seed=21), epochs=20, batch=2048,
              lr=5e-3, band=0.02)
    sc = scenes.torus_fall_scene(200_000, z0=0.105)
    r = sc["radius"]
    a, b = dem.UmScene(sc, dmap), dem.UmScene(sc, dmap)
    counter = torch.zeros(1, dtype=torch.int32, device="cuda")
    steps = 30
    a.update(steps)
    b.update(steps, net=net, skin=2.0 * r, exact_counter=counter)
    dem.check("um update sdf")
    _same(_state(a), _state(b))
    assert 0 < int(counter.item()) < 0.5 * steps * sc["pos"].shape[0]


def test_um_update_with_sdf_tile_culling_equals_exact_map():
    """The same step with the network culling per 32-particle tile (a
    Lipschitz bound measured on held-out pairs): the state of the exact map,
    bit for bit, with fewer exact queries than particles in the map box."""
    from fullc0ntact_gb300 import dem, scenes, sdf
    dmap = dem.DistanceMap.torus(0.3, 0.1, 128, 0.05)
    net = sdf.SdfNet(3, 64, 3, seed=5)
    net.normalize_to(dmap)
    net.train(sdf.samples(dmap, 2_000_000, 0.6, 0.05, seed=21), epochs=20, batch=2048,
              lr=5e-3, band=0.02)
    sc = scenes.torus_fall_scene(200_000, z0=0.105)
    r = sc["radius"]
    skin, _ = sdf.calibrate_skin(net, [dmap], r, shaped=False)
    skin = max(skin, 2.0 * r)
    lip, lip_raw = sdf.calibrate_lipschitz(net, [dmap], shaped=False)
    print("skin", skin, "lipschitz", lip_raw)
    net.set_tile_culling(lip)
    a, b = dem.UmScene(sc, dmap), dem.UmScene(sc, dmap)
    counter = torch.zeros(1, dtype=torch.int32, device="cuda")
    steps = 30
    a.update(steps)
    b.update(steps, net=net, skin=skin, exact_counter=counter)
    dem.check("um update, tile culling")
    _same(_state(a), _state(b))
    assert 0 < int(counter.item()) < 0.9 * steps * sc["pos"].shape[0]
