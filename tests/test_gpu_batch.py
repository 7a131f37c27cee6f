"""Batches of scenes: a batch leaves every scene exactly as stepping the
scene on its own leaves it; graph replay equals direct launches; a
one-scene batch in the reference's [-1,1]^3 box equals fcdemUpdate."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _small_batch(num=12, seed=5):
    from fullc0ntact_gb300 import scenes
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(300), np.log(6000), num)).astype(int)
    return [scenes.batch_scene(int(n), 1000 + k) for k, n in enumerate(sizes)]


@pytest.mark.parametrize("graph", [False, True])
def test_batch_equals_scenes_alone(graph):
    from fullc0ntact_gb300 import dem
    sl = _small_batch()
    b = dem.Batch(sl)
    b.update(5, graph=graph)
    dem.check("batch")
    pos, vel = b.split(b.pos), b.split(b.vel)
    for k, sc in enumerate(sl):
        one = dem.Batch([sc])
        one.update(5, graph=False)
        dem.check("single")
        assert torch.equal(pos[k], one.pos), k
        assert torch.equal(vel[k], one.vel), k


def test_graph_replays_repeatedly():
    from fullc0ntact_gb300 import dem
    sl = _small_batch(6, seed=9)
    a, b = dem.Batch(sl), dem.Batch(sl)
    for _ in range(3):
        a.update(4, graph=True)
        b.update(4, graph=False)
    dem.check()
    assert torch.equal(a.pos, b.pos) and torch.equal(a.vel, b.vel)


def test_one_scene_batch_in_unit_box_equals_update():
    from fullc0ntact_gb300 import dem, scenes
    sc = scenes.packed_scene(30000, grid=128)
    sc["box_lo"] = np.array([-1.0, -1.0, -1.0], np.float32)
    sc["box_hi"] = np.array([1.0, 1.0, 1.0], np.float32)
    b = dem.Batch([sc])
    b.update(4, graph=True)
    ds = dem.DeviceScene(sc)
    ds.update(4)
    dem.check()
    assert torch.equal(b.pos, ds.pos)
    assert torch.equal(b.vel, ds.vel)
