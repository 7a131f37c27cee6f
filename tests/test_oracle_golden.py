"""The CPU oracle against the golden fixtures made by the reference's own
kernel code (tests/golden/gen_golden.py): every stage bit for bit."""
import numpy as np
import pytest

from fcdem_testutil import (GOLDEN_CASES, assert_same_floats, full_cells, load_golden,
                            oracle_params)
from oracle import oracle as O


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_oracle_matches_reference_fixture(name):
    g = load_golden(name)
    P = oracle_params(g["params"])
    st = O.step_stages(P, g["pos0"], g["vel0"], float(g["dt"]))
    np.testing.assert_array_equal(st["pos"].view(np.uint32), g["pos"].view(np.uint32))
    np.testing.assert_array_equal(st["vel_in"].view(np.uint32), g["vel"].view(np.uint32))
    np.testing.assert_array_equal(st["hash"], g["hash"])
    np.testing.assert_array_equal(st["index"], g["index"])
    np.testing.assert_array_equal(st["hash_sorted"], g["hash_sorted"])
    np.testing.assert_array_equal(st["index_sorted"], g["index_sorted"])
    cs = full_cells(g, P.numCells)
    np.testing.assert_array_equal(st["cellStart"], cs)
    np.testing.assert_array_equal(st["cellEnd"][g["cells"]], g["cell_end"])
    np.testing.assert_array_equal(st["sortedPos"], g["pos"][g["index_sorted"]])
    assert_same_floats(st["newVel"], g["new_vel"])


def test_fixture_invariants():
    """Properties the fixtures must have whatever produced them."""
    for name in GOLDEN_CASES:
        g = load_golden(name)
        hs = g["hash_sorted"].astype(np.int64)
        assert np.all(np.diff(hs) >= 0)
        # stable: ties in ascending original index
        same = np.diff(hs) == 0
        assert np.all(np.diff(g["index_sorted"].astype(np.int64))[same] > 0)
        assert sorted(g["index_sorted"].tolist()) == list(range(hs.size))
        # cell ranges tile the sorted array
        order = np.argsort(g["cell_start"])
        starts, ends = g["cell_start"][order], g["cell_end"][order]
        assert starts[0] == 0 and ends[-1] == hs.size
        np.testing.assert_array_equal(starts[1:], ends[:-1])


@pytest.mark.skipif(not O.ref_host_available(), reason="reference host build absent")
@pytest.mark.parametrize("seed", [1, 2, 3])
def test_oracle_matches_reference_code_random(seed):
    """Fresh random scenes (polydisperse-free, the reference has one radius)
    through the reference code built as host code and through the oracle."""
    import ctypes as C
    rng = np.random.default_rng(seed)
    n = int(rng.integers(1, 4000))
    g = int(2 ** rng.integers(2, 6))
    P = O.SimParams()
    P.colliderPos[:] = [-0.5, 0.2, 0.1]
    P.colliderRadius = 0.3
    P.gravity[:] = [0.0, -1e-3, -3e-4]
    P.globalDamping = 0.999
    P.particleRadius = float(rng.uniform(0.01, 0.1))
    P.gridSize[:] = [g, g, g]
    P.numCells = g ** 3
    P.worldOrigin[:] = [-1.0, -1.0, -1.0]
    P.cellSize[:] = [2.0 / g] * 3
    P.numBodies = n
    P.spring, P.damping, P.shear, P.attraction, P.boundaryDamping = 0.5, 0.02, 0.1, 0.003, -0.5
    pos = np.zeros((n, 4), np.float32)
    pos[:, :3] = rng.uniform(-1.1, 1.1, (n, 3))
    pos[:, 3] = 1.0
    vel = np.zeros((n, 4), np.float32)
    vel[:, :3] = rng.uniform(-0.05, 0.05, (n, 3))
    st = O.step_stages(P, pos, vel, 0.3)
    R = O.ref_host()
    p2, v2 = pos.copy(), vel.copy()
    R.fcref_setParameters(C.byref(P))
    R.fcref_integrateSystem(p2, v2, 0.3, n)
    h = np.empty(n, np.uint32)
    x = np.empty(n, np.uint32)
    R.fcref_calcHash(h, x, p2, n)
    R.fcref_sortParticles(h, x, n)
    cs = np.empty(P.numCells, np.uint32)
    ce = np.full(P.numCells, 0xFFFFFFFF, np.uint32)
    sp, sv = np.empty_like(p2), np.empty_like(v2)
    R.fcref_reorderDataAndFindCellStart(cs, ce, sp, sv, h, x, p2, v2, n, P.numCells)
    nv = v2.copy()
    R.fcref_collide(nv, sp, sv, x, cs, ce, n, P.numCells)
    np.testing.assert_array_equal(st["hash_sorted"], h)
    np.testing.assert_array_equal(st["index_sorted"], x)
    np.testing.assert_array_equal(st["cellStart"], cs)
    np.testing.assert_array_equal(st["newVel"].view(np.uint32), nv.view(np.uint32))


def test_oracle_f64_twin_close_to_f32():
    g = load_golden("plain16k")
    P = oracle_params(g["params"])
    st = O.step_stages(P, g["pos0"], g["vel0"], float(g["dt"]))
    nv64 = O.collide_f64(P, st["sortedPos"], st["sortedVel"], st["index_sorted"],
                         st["cellStart"], st["cellEnd"])
    f32 = st["newVel"][:, :3].astype(np.float64) - st["vel_in"][:, :3]
    f64 = nv64[:, :3] - st["vel_in"][:, :3].astype(np.float64)
    scale = np.median(np.linalg.norm(f64, axis=1))
    err = np.linalg.norm(f32 - f64, axis=1) / np.maximum(np.linalg.norm(f64, axis=1), scale)
    assert err.max() < 1e-4


def test_threaded_update_equals_single_thread():
    """The oracle's full update on several host threads (integrate, hash,
    the radix sort, the reorder and collide split into chunks) ends in the
    bits of the single-threaded one, over a few steps of the packed scene."""
    from fullc0ntact_gb300 import scenes
    from fcdem_testutil import oracle_params
    sc = scenes.packed_scene(60_000, grid=64)
    P = oracle_params(bytes(sc["params"]))
    a = (sc["pos"].copy(), sc["vel"].copy())
    b = (sc["pos"].copy(), sc["vel"].copy())
    O.update(P, a[0], a[1], sc["dt"], steps=3, radius_from_w=True, nthreads=1)
    O.update(P, b[0], b[1], sc["dt"], steps=3, radius_from_w=True, nthreads=5)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x.view(np.uint32), y.view(np.uint32))
