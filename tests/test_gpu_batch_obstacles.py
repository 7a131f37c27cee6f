"""Batches with obstacles (config-4 style): the rounded-box map generator
against the analytic rounded box; a batch with one obstacle map per scene
gives the same state as each scene stepped alone; the shape-conditioned
network (11 -> 128 -> 128 -> 1), judged per shape by the exact maps, culls
the map queries without changing any result."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rounded_box_sdf(p, h, rr):
    inner = np.asarray(h, np.float64) - rr
    q = np.abs(p) - inner
    outside = np.linalg.norm(np.maximum(q, 0.0), axis=1)
    inside = np.minimum(q.max(axis=1), 0.0)
    return outside + inside - rr


def test_rounded_box_generator_matches_analytic():
    from fullc0ntact_gb300 import dem
    from oracle import oracle as O
    h, rr = [0.12, 0.27, 0.2], 0.02
    m = dem.DistanceMap.rounded_box(h, rr, 64, 0.05)
    v = m.vertices()
    coords = O.lattice_coords(m.vmin, m.cell_size, m.cells).astype(np.float64)
    sd = _rounded_box_sdf(coords, h, rr)
    assert np.abs(v[:, 0] - sd).max() <= 1e-6
    cp = v[:, 1:].astype(np.float64)
    assert np.abs(_rounded_box_sdf(cp, h, rr)).max() <= 2e-6  # contact points on the surface
    dd = np.linalg.norm(coords - cp, axis=1)  # |distance| = |vertex - contact point|
    assert np.abs(np.abs(v[:, 0]) - dd).max() <= 2e-6


def _small_obstacle_batch(num_scenes=6, n_min=3000, n_max=20000, seed=5):
    from fullc0ntact_gb300 import scenes
    return scenes.batch_obstacle_scenes(num_scenes, n_min, n_max, seed=seed, num_shapes=4)


@pytest.mark.parametrize("graph", [False, True])
def test_obstacle_batch_equals_each_scene_alone(graph):
    from fullc0ntact_gb300 import dem, sdf
    scs, obs, shape = _small_obstacle_batch()
    maps = sdf.obstacle_maps(obs, 64)
    b = dem.Batch(scs)
    b.set_obstacles(maps, shape)
    steps = 25
    b.update(steps, graph=graph)
    dem.check("batch")
    assert b.exact_queries() > 0  # the spheres reach their obstacles
    for k, sc in enumerate(scs):
        one = dem.Batch([sc])
        one.set_obstacles(maps, [shape[k]])
        one.update(steps, graph=False)
        dem.check("scene")
        for x, y in ((b.split(b.pos)[k], one.pos), (b.split(b.vel)[k], one.vel)):
            np.testing.assert_array_equal(x.cpu().numpy().view(np.uint32),
                                          y.cpu().numpy().view(np.uint32))


def test_shape_network_judged_by_maps_and_culling_is_exact():
    from fullc0ntact_gb300 import dem, sdf
    scs, obs, shape = _small_obstacle_batch(num_scenes=8, seed=6)
    maps = sdf.obstacle_maps(obs, 128)
    net, loss = sdf.shape_net(maps)
    print("shape net loss", loss)
    assert loss < 2e-4
    r_max = 1.0 / 256.0
    # the skin from one held-out set, checked on another
    skin, p_max = sdf.calibrate_skin(net, maps, r_max, seed=300)
    print("skin", skin, "p_max", p_max)
    assert skin < 8.0 * r_max
    for k, m in enumerate(maps):
        val, sh = sdf.samples(m, 200_000, 0.5, 0.03, seed=500 + k, shape=k)
        pred = net.infer(val, sh)
        d = val[:, 3]
        near = d.abs() < 0.02
        err = float((pred - d)[near].abs().max())
        print(k, "max err near", err, "bad", int(((d < r_max) & (pred > skin)).sum()))
        assert int(((d < r_max) & (pred > skin)).sum()) == 0, k
    a, b = dem.Batch(scs), dem.Batch(scs)
    a.set_obstacles(maps, shape)
    b.set_obstacles(maps, shape, net=net, skin=skin)
    steps = 40
    a.update(steps, graph=True)
    b.update(steps, graph=True)
    dem.check("batch neural")
    np.testing.assert_array_equal(a.pos.cpu().numpy().view(np.uint32),
                                  b.pos.cpu().numpy().view(np.uint32))
    np.testing.assert_array_equal(a.vel.cpu().numpy().view(np.uint32),
                                  b.vel.cpu().numpy().view(np.uint32))
    ea, eb = a.exact_queries(), b.exact_queries()
    print("exact queries exact/neural", ea, eb)
    assert 0 < eb < 0.7 * ea, (ea, eb)


def test_graph_records_again_after_the_network_changes():
    """A batch replayed from a CUDA graph holds the network's normalisation
    and BF16 weights of its recording; after the network is given new
    parameters the next update records again.  Here the new parameters make
    it predict a distance far above the skin everywhere, so the map queries
    all but stop (the results then differ: the test is about the recording,
    not about culling)."""
    from fullc0ntact_gb300 import dem, sdf
    scs, obs, shape = _small_obstacle_batch(num_scenes=3, n_min=3000, n_max=6000, seed=12)
    maps = sdf.obstacle_maps(obs, 64)
    net = sdf.SdfNet(3 + len(maps), 128, 2, seed=3)
    net.set_normalization([0.0, 0.0, 0.0], [2.0, 2.0, 2.0], 0.5)
    b = dem.Batch(scs)
    b.set_obstacles(maps, shape, net=net, skin=10.0)  # nothing above the skin: no culling
    b.update(30, graph=True)
    b.update(10, graph=True)
    b.exact_queries(reset=True)
    b.update(10, graph=True)  # replay
    dem.check("replay")
    before = b.exact_queries(reset=True)
    assert before > 0
    p = np.zeros(net.num_params, np.float32)
    p[-1] = 1e6  # output bias: every prediction far above the skin
    net.set_params(p)
    b.update(10, graph=True)
    dem.check("after the change")
    after = b.exact_queries(reset=True)
    print("exact queries per 10 steps before / after", before, after)
    assert after < 0.2 * before


def test_tile_culling_is_exact_and_queries_less():
    """Culling per tile (fcdemSdfSetTileCulling): the shape network runs once
    per 32-slot tile at the centre of the tile's particles in the map box,
    with a Lipschitz bound measured on held-out pairs.  40 batched steps end
    in the bits of the exact maps, with fewer exact queries."""
    from fullc0ntact_gb300 import dem, sdf
    scs, obs, shape = _small_obstacle_batch(num_scenes=8, seed=6)
    maps = sdf.obstacle_maps(obs, 128)
    net, loss = sdf.shape_net(maps)
    r_max = 1.0 / 256.0
    skin, _ = sdf.calibrate_skin(net, maps, r_max, seed=300)
    lip, lip_raw = sdf.calibrate_lipschitz(net, maps)
    print("skin", skin, "lipschitz", lip_raw, "used", lip)
    assert 0.5 < lip_raw < 4.0  # a distance field's slope is 1
    net.set_tile_culling(lip)
    a, b = dem.Batch(scs), dem.Batch(scs)
    a.set_obstacles(maps, shape)
    b.set_obstacles(maps, shape, net=net, skin=skin)
    steps = 40
    a.update(steps, graph=True)
    b.update(steps, graph=True)
    dem.check("batch, tile culling")
    np.testing.assert_array_equal(a.pos.cpu().numpy().view(np.uint32),
                                  b.pos.cpu().numpy().view(np.uint32))
    np.testing.assert_array_equal(a.vel.cpu().numpy().view(np.uint32),
                                  b.vel.cpu().numpy().view(np.uint32))
    ea, eb = a.exact_queries(), b.exact_queries()
    print("exact queries exact/tile-culled", ea, eb)
    assert 0 < eb < ea, (ea, eb)


def test_tile_culling_with_scenes_without_obstacles_and_shared_tiles():
    """Culling per tile where scenes end inside a 32-slot tile (tiles with
    particles of two obstacles are never culled) and some scenes have no
    obstacle (shape -1): the bits of the exact maps, plain and from a graph."""
    from fullc0ntact_gb300 import dem, sdf
    scs, obs, shape = _small_obstacle_batch(num_scenes=6, n_min=1000, n_max=5000, seed=9)
    shape = [s if k % 3 != 1 else -1 for k, s in enumerate(shape)]
    maps = sdf.obstacle_maps(obs, 64)
    net, _ = sdf.shape_net(maps)
    r_max = 1.0 / 256.0
    skin, _ = sdf.calibrate_skin(net, maps, r_max, seed=301)
    lip, _ = sdf.calibrate_lipschitz(net, maps, pairs_per_map=200_000)
    net.set_tile_culling(lip)
    for graph in (False, True):
        a, b = dem.Batch(scs), dem.Batch(scs)
        a.set_obstacles(maps, shape)
        b.set_obstacles(maps, shape, net=net, skin=skin)
        a.update(30, graph=graph)
        b.update(30, graph=graph)
        dem.check("tile culling, mixed tiles")
        for x, y in ((a.pos, b.pos), (a.vel, b.vel)):
            np.testing.assert_array_equal(x.cpu().numpy().view(np.uint32),
                                          y.cpu().numpy().view(np.uint32))
        assert b.exact_queries() <= a.exact_queries()
