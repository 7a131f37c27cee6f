"""Whole updates: the fused fcdemUpdate leaves the same state as the five
reference-named calls; the C++ ParticleSystem drives them; multi-step runs
agree with the oracle in energy, momentum and contact statistics."""
import numpy as np
import pytest
import torch

from fcdem_testutil import oracle_params

pytestmark = pytest.mark.gpu


def _state(ds):
    return (ds.pos.cpu().numpy().copy(), ds.vel.cpu().numpy().copy(),
            ds.hash.cpu().numpy().copy(), ds.index.cpu().numpy().copy(),
            ds.sorted_pos.cpu().numpy().copy(), ds.sorted_vel.cpu().numpy().copy())


@pytest.mark.parametrize("pipeline", [0, 1])
@pytest.mark.parametrize("poly", [False, True])
@pytest.mark.parametrize("steps", [1, 2, 5])
def test_fused_update_equals_staged(pipeline, poly, steps):
    """Both fcdemUpdate pipelines (0: radix sort + fill + reorder, 1: cell
    counting sort with stable fix-up) against the five staged calls."""
    from fullc0ntact_gb300 import dem, scenes
    sc = (scenes.random_box(5000, grid=(32, 32, 32), radius=1.0 / 24.0, seed=3, poly=True)
          if poly else scenes.lattice_scene(4096))
    a, b = dem.DeviceScene(sc), dem.DeviceScene(sc)
    for _ in range(steps):
        a.stages()
    dem.lib.fcdemSetUpdatePipeline(pipeline)
    try:
        b.update(steps)
    finally:
        dem.lib.fcdemSetUpdatePipeline(1)
    dem.check("update")
    for x, y in zip(_state(a), _state(b)):
        np.testing.assert_array_equal(x.view(np.uint32), y.view(np.uint32))
    cs_a, cs_b = a.cell_start.cpu().numpy(), b.cell_start.cpu().numpy()
    np.testing.assert_array_equal(cs_a, cs_b)
    ne = cs_a != -1
    np.testing.assert_array_equal(a.cell_end.cpu().numpy()[ne], b.cell_end.cpu().numpy()[ne])


def test_particle_system_class():
    """The headless ParticleSystem with the reference's defaults."""
    from fullc0ntact_gb300 import dem
    ps = dem.ParticleSystem(4096, (64, 64, 64))
    p = ps.params
    assert abs(p.particleRadius - 1.0 / 16.0) < 1e-9 and p.numCells == 64 ** 3
    p.particleRadius = 1.0 / 64.0
    p.cellSize[:] = [1.0 / 32.0] * 3
    ps.reset(dem.ParticleSystem.CONFIG_GRID)
    pos0 = ps.get_array(dem.ParticleSystem.POSITION)
    assert np.all(pos0[:, 3] == 1.0) and pos0[:, :3].min() > -1.0
    ps.set_fused_update(False)
    ps.update(0.5)
    ps.update(0.5)
    staged = ps.get_array(dem.ParticleSystem.VELOCITY)
    ps2 = dem.ParticleSystem(4096, (64, 64, 64))
    ps2.params.particleRadius = 1.0 / 64.0
    ps2.params.cellSize[:] = [1.0 / 32.0] * 3
    ps2.reset(dem.ParticleSystem.CONFIG_GRID)
    ps2.update_steps(0.5, 2)
    fused = ps2.get_array(dem.ParticleSystem.VELOCITY)
    np.testing.assert_array_equal(staged, fused)
    assert ps2.dump_grid() >= 1
    dem.check("ParticleSystem")


def _stats(pos, vel, radius, gz=-3e-4):
    v = vel[:, :3].astype(np.float64)
    ke = 0.5 * np.sum(v * v)
    pe = -gz * np.sum(pos[:, 2].astype(np.float64) + 1.0)
    mom = v.sum(axis=0)
    return ke, pe, mom


def test_multistep_statistics_match_oracle():
    """Trajectories are chaotic, so 50 steps are compared by total energy,
    momentum and contact count, not particle by particle."""
    from fullc0ntact_gb300 import dem, scenes
    from oracle import oracle as O
    sc = scenes.lattice_scene(8192)
    ds = dem.DeviceScene(sc)
    ds.update(50)
    dem.check()
    P = oracle_params(bytes(sc["params"]))
    pos, vel = sc["pos"].copy(), sc["vel"].copy()
    O.update(P, pos, vel, sc["dt"], steps=50)
    g_pos, g_vel = ds.pos.cpu().numpy(), ds.vel.cpu().numpy()
    ke_g, pe_g, mom_g = _stats(g_pos, g_vel, P.particleRadius)
    ke_o, pe_o, mom_o = _stats(pos, vel, P.particleRadius)
    assert abs(ke_g - ke_o) <= 0.02 * ke_o + 1e-12
    assert abs(pe_g - pe_o) <= 1e-3 * abs(pe_o)
    assert np.all(np.abs(mom_g - mom_o) <= 0.05 * np.abs(mom_o).max() + 1e-9)
    # contact count of the final configuration
    def contacts(p):
        h, x = O.calc_hash(P, p)
        hs, xs = O.sort_pairs(h, x)
        cs, ce, sp, sv = O.reorder(hs, xs, p, vel, P.numCells)
        nv = O.collide(P, sp, sv, xs, cs, ce)
        return int(np.count_nonzero(np.any(nv[:, :3] != vel[:, :3], axis=1)))
    c_g, c_o = contacts(g_pos), contacts(pos)
    assert abs(c_g - c_o) <= 0.02 * c_o


def test_stream_selection():
    from fullc0ntact_gb300 import dem, scenes
    sc = scenes.lattice_scene(2048)
    a, b = dem.DeviceScene(sc), dem.DeviceScene(sc)
    a.update(3)
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        dem.set_stream(s)
        b.update(3)
        dem.set_stream(None)
    s.synchronize()
    dem.check()
    np.testing.assert_array_equal(a.vel.cpu().numpy(), b.vel.cpu().numpy())


def test_counting_pipeline_on_packed_scene_and_crowded_cells():
    """The counting sort's within-cell fix-up on a scene with crowded cells
    (40 particles in one cell) and on a packed polydisperse scene."""
    from fullc0ntact_gb300 import dem, scenes
    for sc in (scenes.random_box(3000, grid=(8, 8, 8), radius=0.02, cell=0.25, seed=4),
               scenes.packed_scene(100_000, grid=128)):
        sc["pos"][:40, :3] = 0.01 + 0.001 * np.arange(40, dtype=np.float32)[:, None]
        a, b = dem.DeviceScene(sc), dem.DeviceScene(sc)
        for _ in range(3):
            a.stages()
        b.update(3)
        dem.check("update")
        for x, y in zip(_state(a), _state(b)):
            np.testing.assert_array_equal(x.view(np.uint32), y.view(np.uint32))


@pytest.mark.parametrize("n,kind", [(6000, "box8"), (100_000, "packed"), (1_000_000, "box128")])
def test_counting_pipeline_cells_above_rerank_limit(n, kind):
    """Cells holding more than the per-slot re-rank handles (1,024) are
    ranked by particle index in one CTA each: with a bitmap of the members'
    indices when their span is at most 16 words per member, else with a
    block radix sort (n = 100,000 needs three 8-bit passes, n = 6,000 two).
    At n = 1,000,000 the 3,000-member cell takes the bitmap and the 1,500-
    and 1,025-member cells the sort; at the smaller n every cell takes the
    bitmap.  The result stays identical to the staged radix-sort path."""
    from fullc0ntact_gb300 import dem, scenes
    if kind == "box8":
        sc = scenes.random_box(n, grid=(8, 8, 8), radius=0.02, cell=0.25, seed=11)
    elif kind == "box128":
        sc = scenes.random_box(n, grid=(128, 128, 128), radius=1.0 / 128.0, seed=13)
    else:
        sc = scenes.packed_scene(n, grid=128)
    rng = np.random.default_rng(5)
    cell = float(sc["params"].cellSize[0])
    origin = np.array([sc["params"].worldOrigin[k] for k in range(3)], np.float32)
    # three crowded cells: 3,000 / 1,500 / 1,025 members (two of them in the
    # same neighbourhood), drawn from scattered particle indices
    picks = rng.permutation(n)
    start = 0
    for count, c in ((3000, (3, 3, 3)), (1500, (4, 3, 3)), (1025, (6, 6, 6))):
        idx = picks[start:start + count]
        start += count
        lo = origin + np.array(c, np.float32) * cell
        sc["pos"][idx, :3] = lo + rng.uniform(0.2, 0.8, (count, 3)).astype(np.float32) * cell
    a, b = dem.DeviceScene(sc), dem.DeviceScene(sc)
    for _ in range(2):
        a.stages()
    b.update(2)
    dem.check("update")
    for x, y in zip(_state(a), _state(b)):
        np.testing.assert_array_equal(x.view(np.uint32), y.view(np.uint32))


def test_counting_pipeline_many_tiles():
    """A 512^3 grid (134M cells, 32,769 tiles of 4,096 cells): the tile
    prefix runs as block scans plus block offsets; the fused update still
    equals the staged path, cell tables included."""
    from fullc0ntact_gb300 import dem, scenes
    sc = scenes.random_box(40_000, grid=(512, 512, 512), radius=1.0 / 256.0,
                           cell=1.0 / 256.0, seed=12)
    a, b = dem.DeviceScene(sc), dem.DeviceScene(sc)
    for _ in range(3):
        a.stages()
    b.update(3)
    dem.check("update")
    for x, y in zip(_state(a), _state(b)):
        np.testing.assert_array_equal(x.view(np.uint32), y.view(np.uint32))
    sa, sb = dem.u32(a.cell_start), dem.u32(b.cell_start)
    np.testing.assert_array_equal(sa, sb)
    occ = sa != 0xFFFFFFFF
    np.testing.assert_array_equal(dem.u32(a.cell_end)[occ], dem.u32(b.cell_end)[occ])


@pytest.mark.parametrize("crowd", [1, 0])
def test_staged_rows_with_many_contacts_equal_staged_calls(crowd):
    """Dense scenes where the lanes of a warp fall out of step inside a
    neighbour row: about 60 contacts per sphere (several queue drains per
    row), warps that mix spheres of edge columns (rows walked cell by cell)
    with interior ones (rows copied to shared memory), and -- with the
    crowded-neighbourhood kernel switched off -- collapsed cells whose rows
    are too long to copy.  The fused update, whose collide copies each row
    once per warp, against the reference-named stages, whose collide reads
    every partner from global memory: the same bits over four steps."""
    from fullc0ntact_gb300 import dem, scenes
    from test_gpu_collide_paths import _crowded_scene
    dem.lib.fcdemSetCrowdPath(crowd)
    try:
        for sc in (scenes.random_box(60000, grid=(16, 16, 16), radius=1.0 / 16.0, seed=14),
                   _crowded_scene("packed")):
            a, b = dem.DeviceScene(sc), dem.DeviceScene(sc)
            for _ in range(4):
                a.stages()
            b.update(4)
            dem.check("update")
            for x, y in zip(_state(a), _state(b)):
                np.testing.assert_array_equal(x.view(np.uint32), y.view(np.uint32))
    finally:
        dem.lib.fcdemSetCrowdPath(1)


@pytest.mark.parametrize("n", [1, 2, 31, 33, 129, 1000])
def test_fused_update_with_partial_warps(n):
    """Particle counts that leave the last warp, or the only one, partly
    empty (the collide's lane mask, its row copies and the crowded lists
    then cover fewer than 32 lanes): five fused updates against the staged
    calls, in a box small enough that the particles touch."""
    from fullc0ntact_gb300 import dem, scenes
    sc = scenes.random_box(n, grid=(8, 8, 8), radius=0.1, cell=0.25, seed=n, poly=(n % 2 == 1))
    a, b = dem.DeviceScene(sc), dem.DeviceScene(sc)
    for _ in range(5):
        a.stages()
    b.update(5)
    dem.check("partial warps")
    for x, y in zip(_state(a), _state(b)):
        np.testing.assert_array_equal(x.view(np.uint32), y.view(np.uint32))
