"""The collide kernels give bit-identical results: the per-thread kernel with
global reads, the kernel with shared-memory tiles staged by bulk copies, and
the kernel for crowded neighbourhoods, on scenes that exercise staged tiles,
multi-row tiles, x-wrapping windows, crowded cells, inert particles and the
polydisperse mode."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run(sc, path, steps):
    from fullc0ntact_gb300 import dem
    dem.lib.fcdemSetCollidePath(path)
    try:
        ds = dem.DeviceScene(sc)
        ds.stages()
        if steps > 1:
            ds.update(steps - 1)
        dem.check("collide path %d" % path)
        return ds.pos.cpu().numpy(), ds.vel.cpu().numpy()
    finally:
        dem.lib.fcdemSetCollidePath(-1)


@pytest.mark.parametrize("case", ["packed", "lattice", "wrap", "random_poly", "sparse"])
def test_tiled_equals_global(case):
    from fullc0ntact_gb300 import scenes
    if case == "packed":
        sc = scenes.packed_scene(200_000, grid=128)
    elif case == "lattice":
        sc = scenes.lattice_scene(16384)
    elif case == "wrap":  # particles across the whole x range: windows wrap
        sc = scenes.random_box(30000, grid=(32, 32, 32), radius=1.0 / 32.0, seed=8)
    elif case == "random_poly":
        sc = scenes.random_box(30000, grid=(64, 64, 64), radius=1.0 / 64.0, seed=9, poly=True)
    else:  # few particles per row: many row groups per tile
        sc = scenes.random_box(3000, grid=(64, 64, 64), radius=1.0 / 64.0, seed=10)
    a = _run(sc, 0, 3)
    b = _run(sc, 1, 3)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x.view(np.uint32), y.view(np.uint32))


def _run_cull(sc, on, steps):
    from fullc0ntact_gb300 import dem
    dem.lib.fcdemSetCellCulling(int(on))
    try:
        ds = dem.DeviceScene(sc)
        ds.stages()
        if steps > 1:
            ds.update(steps - 1)
        dem.check("cell culling %d" % on)
        return ds.pos.cpu().numpy(), ds.vel.cpu().numpy()
    finally:
        dem.lib.fcdemSetCellCulling(1)


@pytest.mark.parametrize("case", ["packed", "lattice", "wrap", "random_poly", "small_grid"])
def test_cell_culling_is_exact(case):
    from fullc0ntact_gb300 import scenes
    if case == "packed":
        sc = scenes.packed_scene(200_000, grid=128)
    elif case == "lattice":
        sc = scenes.lattice_scene(16384)
    elif case == "wrap":
        sc = scenes.random_box(30000, grid=(32, 32, 32), radius=1.0 / 64.0, seed=8)
    elif case == "random_poly":  # particleRadius bounds the radii in w
        sc = scenes.random_box(30000, grid=(64, 64, 64), radius=1.0 / 64.0, seed=9, poly=True)
    else:  # grid too small for culling: it must switch itself off
        sc = scenes.random_box(2000, grid=(2, 4, 4), radius=0.1, cell=0.5, seed=11)
    a = _run_cull(sc, False, 4)
    b = _run_cull(sc, True, 4)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x.view(np.uint32), y.view(np.uint32))


def test_radius_bound_violation_is_reported():
    from fullc0ntact_gb300 import _native, dem, scenes
    sc = scenes.random_box(5000, grid=(64, 64, 64), radius=1.0 / 64.0, seed=12, poly=True)
    sc["pos"][17, 3] = 2.0 / 64.0  # above particleRadius
    ds = dem.DeviceScene(sc)
    ds.stages()
    with pytest.raises(_native.FcdemError, match="radius"):
        dem.check()


def _crowded_scene(kind):
    """Scenes with collapsed cells: thousands of particles in a few cells, the
    cells around them sparse or crowded too."""
    from fullc0ntact_gb300 import scenes
    if kind == "mono":
        sc = scenes.random_box(20000, grid=(16, 16, 16), radius=1.0 / 16.0, seed=21)
    elif kind == "poly":
        sc = scenes.random_box(20000, grid=(16, 16, 16), radius=1.0 / 16.0, seed=22, poly=True)
    else:  # packed polydisperse scene with three collapsed cells
        sc = scenes.packed_scene(100_000, grid=128)
    rng = np.random.default_rng(23)
    cell = float(sc["params"].cellSize[0])
    origin = np.array([sc["params"].worldOrigin[k] for k in range(3)], np.float32)
    n = sc["pos"].shape[0]
    picks = rng.permutation(n)
    start = 0
    for count, c in ((2500, (5, 5, 5)), (700, (6, 5, 5)), (300, (9, 9, 9)), (90, (12, 3, 7))):
        idx = picks[start:start + count]
        start += count
        lo = origin + np.array(c, np.float32) * cell
        sc["pos"][idx, :3] = lo + rng.uniform(0.05, 0.95, (count, 3)).astype(np.float32) * cell
    return sc


def _run_crowd(sc, on, steps, pipeline=1):
    from fullc0ntact_gb300 import dem
    dem.lib.fcdemSetCrowdPath(int(on))
    dem.lib.fcdemSetUpdatePipeline(pipeline)
    try:
        ds = dem.DeviceScene(sc)
        ds.stages()
        if steps > 1:
            ds.update(steps - 1)
        dem.check("crowd path %d" % on)
        return ds.pos.cpu().numpy(), ds.vel.cpu().numpy(), ds.hash.cpu().numpy()
    finally:
        dem.lib.fcdemSetCrowdPath(1)
        dem.lib.fcdemSetUpdatePipeline(1)


@pytest.mark.parametrize("kind", ["mono", "poly", "packed"])
@pytest.mark.parametrize("pipeline", [0, 1])
def test_crowd_path_is_exact(kind, pipeline):
    """The warp-per-group kernel for crowded neighbourhoods gives results
    bit-identical to the one-thread-per-particle kernel, through the
    reference-named stages and both fcdemUpdate pipelines."""
    sc = _crowded_scene(kind)
    a = _run_crowd(sc, True, 3, pipeline)
    b = _run_crowd(sc, False, 3, pipeline)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x.view(np.uint32), y.view(np.uint32))


def _inert_scene():
    """Packed polydisperse scene with particles that take part in no pair
    term: 3,000 with NaN positions (they share one cell, a crowded
    neighbourhood), 300 with one NaN coordinate, and 40 spheres of equal
    radius at one point (coincident: dist = 0, their normals are NaN)."""
    from fullc0ntact_gb300 import scenes
    sc = scenes.packed_scene(100_000, grid=128)
    rng = np.random.default_rng(31)
    picks = rng.permutation(sc["pos"].shape[0])
    sc["pos"][picks[:3000], :3] = np.float32(np.nan)
    for k, idx in enumerate(np.array_split(picks[3000:3300], 3)):
        sc["pos"][idx, k] = np.float32(np.nan)
    same = picks[3300:3340]
    sc["pos"][same, :3] = np.float32(0.25)
    sc["pos"][same, 3] = np.float32(sc["params"].particleRadius)
    sc["vel"][same, :3] = np.float32(0.0)  # still coincident after the integrate
    return sc


def test_inert_particles_match_oracle():
    """Particles with a NaN coordinate are skipped by collide (their force is
    +0.0 and they give their partners nothing); the oracle walks them like
    every other particle.  One update through the reference-named stages:
    hashes and order bit for bit, new velocities within the 1e-5 bar with
    NaN exactly where the oracle has NaN."""
    from fullc0ntact_gb300 import dem
    from oracle import oracle as O
    from fcdem_testutil import REL_TOL, force_floor, oracle_params, rel_err_vec
    sc = _inert_scene()
    ds = dem.DeviceScene(sc)
    ds.stages()
    dem.check("stages with inert particles")
    st = O.step_stages(oracle_params(bytes(sc["params"])), sc["pos"], sc["vel"], sc["dt"],
                       radius_from_w=True)
    np.testing.assert_array_equal(ds.hash.cpu().numpy().view(np.uint32), st["hash_sorted"])
    np.testing.assert_array_equal(ds.index.cpu().numpy().view(np.uint32), st["index_sorted"])
    out = ds.vel.cpu().numpy()
    np.testing.assert_array_equal(np.isnan(out[:, :3]), np.isnan(st["newVel"][:, :3]))
    assert int(np.isnan(out[:, 0]).sum()) >= 40  # the coincident spheres
    # a particle with a NaN coordinate keeps its velocity (force +0.0)
    inert = np.isnan(st["pos"][:, :3]).any(axis=1)
    assert int(inert.sum()) == 3300
    keep = st["vel_in"][inert, :3] + np.float32(0.0)
    np.testing.assert_array_equal(out[inert, :3].view(np.uint32), keep.view(np.uint32))
    f_ref = st["newVel"][:, :3].astype(np.float64) - st["vel_in"][:, :3]
    f_gpu = out[:, :3].astype(np.float64) - st["vel_in"][:, :3]
    assert rel_err_vec(out, st["newVel"], 1e-6).max() <= REL_TOL
    assert rel_err_vec(f_gpu, f_ref, force_floor(f_ref)).max() <= REL_TOL


@pytest.mark.parametrize("pipeline", [0, 1])
def test_inert_particles_identical_on_every_path(pipeline):
    """Five fused updates of the scene with inert particles: the crowded
    kernel (which skips chunks of inert partners) and the per-thread kernel
    give the same bits."""
    sc = _inert_scene()
    a = _run_crowd(sc, True, 5, pipeline)
    b = _run_crowd(sc, False, 5, pipeline)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x.view(np.uint32), y.view(np.uint32))


@pytest.mark.parametrize("limit", [128, 2048])
def test_crowd_limit_does_not_change_results(limit):
    """The neighbourhood size above which a particle goes to the crowded
    kernel (fcdemSetCrowdLimit) moves work between the two kernels only:
    three fused updates of the packed scene with crowded cells end in the
    same bits at the default limit (512) and at `limit`."""
    from fullc0ntact_gb300 import dem
    sc = _crowded_scene("packed")
    a = _run_crowd(sc, True, 3)
    dem.lib.fcdemSetCrowdLimit(limit)
    try:
        b = _run_crowd(sc, True, 3)
    finally:
        dem.lib.fcdemSetCrowdLimit(0)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x.view(np.uint32), y.view(np.uint32))



def test_collide_configurations_give_identical_results():
    """Three fused updates of the packed scene with collapsed cells under
    collide configurations that differ in crowd limit, persistent-grid width
    and row staging: the same bits as the default configuration."""
    from fullc0ntact_gb300 import dem
    sc = _crowded_scene("packed")
    dem.lib.fcdemSetCollideConfig(-1)
    ref = _run_crowd(sc, True, 3)
    try:
        for k in (0, 1, 7, 15, 22, 29):
            dem.lib.fcdemSetCollideConfig(k)
            got = _run_crowd(sc, True, 3)
            for x, y in zip(ref, got):
                np.testing.assert_array_equal(x.view(np.uint32), y.view(np.uint32))
    finally:
        dem.lib.fcdemSetCollideConfig(-1)


def test_collide_autotuner_keeps_the_state_and_the_results():
    """fcdemAutotuneCollide on the packed scene with collapsed cells: it returns
    a configuration index and a step time, puts pos and vel back as they were,
    and the next update under the chosen configuration gives the bits of the
    default one."""
    import torch
    from fullc0ntact_gb300 import dem
    sc = _crowded_scene("packed")
    ds = dem.DeviceScene(sc)
    pos0, vel0 = ds.pos.clone(), ds.vel.clone()
    k, ms = ds.autotune_collide()
    try:
        assert 0 <= k < 30 and ms > 0.0
        assert torch.equal(ds.pos.view(torch.int32), pos0.view(torch.int32))
        assert torch.equal(ds.vel.view(torch.int32), vel0.view(torch.int32))
        ds.update(2)
        dem.check("update after autotune")
        tuned = (ds.pos.cpu().numpy(), ds.vel.cpu().numpy())
    finally:
        dem.lib.fcdemSetCollideConfig(-1)
    ds2 = dem.DeviceScene(sc)
    ds2.update(2)
    dem.check("update, default configuration")
    for x, y in zip(tuned, (ds2.pos.cpu().numpy(), ds2.vel.cpu().numpy())):
        np.testing.assert_array_equal(x.view(np.uint32), y.view(np.uint32))
