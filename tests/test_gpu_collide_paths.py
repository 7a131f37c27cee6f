"""The two collide kernels (global reads / shared-memory tiles staged by bulk
copies) give bit-identical results, on scenes that exercise staged tiles,
multi-row tiles, x-wrapping windows and the polydisperse mode."""
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
        sc = scenes.config1(200_000, grid=128)
    elif case == "lattice":
        sc = scenes.config0(16384)
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
        sc = scenes.config1(200_000, grid=128)
    elif case == "lattice":
        sc = scenes.config0(16384)
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
