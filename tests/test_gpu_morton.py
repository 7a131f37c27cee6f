"""Morton cell keys (fcdemSetCellOrder(1)).  The sorted order differs from
the reference's linear order, so the checks are: every particle's Morton key
decodes to its linear hash; the members of each cell, in their order, are
the same; cell lengths are equal; and positions, velocities and forces are
bit-identical to linear order, on the staged stages, both fused pipelines,
the unified-memory step with a map and a crowded scene."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _demorton(k, bits=10):
    k = k.astype(np.int64)
    x = np.zeros_like(k)
    y = np.zeros_like(k)
    z = np.zeros_like(k)
    for b in range(bits):
        x |= ((k >> (3 * b)) & 1) << b
        y |= ((k >> (3 * b + 1)) & 1) << b
        z |= ((k >> (3 * b + 2)) & 1) << b
    return x, y, z


def _run(sc, morton, fn):
    from fullc0ntact_gb300 import dem
    dem.lib.fcdemSetCellOrder(int(morton))
    try:
        return fn(sc)
    finally:
        dem.lib.fcdemSetCellOrder(0)


def _same_bits(a, b):
    np.testing.assert_array_equal(np.asarray(a).view(np.uint32), np.asarray(b).view(np.uint32))


@pytest.mark.parametrize("kind", ["lattice", "packed"])
def test_staged_stages_morton_vs_linear(kind):
    from fullc0ntact_gb300 import dem, scenes
    sc = scenes.lattice_scene(16384) if kind == "lattice" else scenes.packed_scene(100_000, grid=128)

    def stages(sc):
        ds = dem.DeviceScene(sc)
        ds.stages()
        dem.check("stages")
        return dict(pos=ds.pos.cpu().numpy(), vel=ds.vel.cpu().numpy(),
                    hash=dem.u32(ds.hash), index=dem.u32(ds.index),
                    start=dem.u32(ds.cell_start), end=dem.u32(ds.cell_end))

    lin = _run(sc, False, stages)
    mor = _run(sc, True, stages)
    _same_bits(lin["pos"], mor["pos"])
    _same_bits(lin["vel"], mor["vel"])
    g = int(sc["params"].gridSize[0])
    x, y, z = _demorton(mor["hash"])
    lin_of_mor = (z * g + y) * g + x
    # each particle's Morton key decodes to its linear hash
    lin_hash_of = np.empty(len(lin["index"]), np.int64)
    lin_hash_of[lin["index"]] = lin["hash"]
    np.testing.assert_array_equal(lin_of_mor, lin_hash_of[mor["index"]])
    # a stable sort of the Morton order by linear cell gives the linear order:
    # the same members of every cell, in the same order
    order = np.argsort(lin_of_mor, kind="stable")
    np.testing.assert_array_equal(mor["index"][order], lin["index"])
    # cell lengths
    occ = lin["start"] != 0xFFFFFFFF
    cells = np.nonzero(occ)[0]
    cx, cy, cz = cells % g, (cells // g) % g, cells // (g * g)
    mk = np.zeros_like(cells)
    for b in range(10):
        mk |= ((cx >> b) & 1) << (3 * b) | ((cy >> b) & 1) << (3 * b + 1) | \
              ((cz >> b) & 1) << (3 * b + 2)
    np.testing.assert_array_equal(lin["end"][cells] - lin["start"][cells],
                                  mor["end"][mk] - mor["start"][mk])
    assert int((mor["start"] != 0xFFFFFFFF).sum()) == len(cells)


@pytest.mark.parametrize("pipeline", [0, 1])
def test_fused_update_morton_vs_linear(pipeline):
    from fullc0ntact_gb300 import dem, scenes
    sc = scenes.packed_scene(200_000, grid=128)

    def upd(sc):
        dem.lib.fcdemSetUpdatePipeline(pipeline)
        try:
            ds = dem.DeviceScene(sc)
            ds.update(6)
            dem.check("update")
            return ds.pos.cpu().numpy(), ds.vel.cpu().numpy()
        finally:
            dem.lib.fcdemSetUpdatePipeline(1)

    for a, b in zip(_run(sc, False, upd), _run(sc, True, upd)):
        _same_bits(a, b)


def test_um_update_with_map_and_crowded_cells_morton_vs_linear():
    from fullc0ntact_gb300 import dem, scenes
    dmap = dem.DistanceMap.torus(0.3, 0.1, 128, 0.05)
    sc = scenes.torus_fall_scene(80_000, z0=0.09)
    # a collapsed cell and its neighbourhood (the crowd path)
    rng = np.random.default_rng(3)
    idx = rng.permutation(sc["pos"].shape[0])[:3000]
    sc["pos"][idx, :3] = np.array([0.5, 0.5, 0.3], np.float32) + \
        rng.uniform(0.0, 1.0 / 128.0, (3000, 3)).astype(np.float32)

    def upd(sc):
        us = dem.UmScene(sc, dmap)
        us.update(5)
        dem.check("um update")
        return us.pos.cpu().numpy(), us.vel.cpu().numpy(), us.force.cpu().numpy()

    for a, b in zip(_run(sc, False, upd), _run(sc, True, upd)):
        _same_bits(a, b)
