"""sortParticles: the onesweep radix sort against a stable CPU sort, on the
key distributions the step produces and on edge cases."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _sort_gpu(keys, vals, num_cells):
    from fullc0ntact_gb300 import dem
    from fullc0ntact_gb300.params import make_params
    g = 1
    while g ** 3 < num_cells:
        g *= 2
    P = make_params(len(keys), (g, g, g), 0.01)
    P.numCells = num_cells
    dem.set_parameters(P)
    k = torch.from_numpy(keys.view(np.int32).copy()).cuda()
    v = torch.from_numpy(vals.view(np.int32).copy()).cuda()
    dem.sort_particles(k, v, len(keys))
    dem.check("sortParticles")
    return k.cpu().numpy().view(np.uint32), v.cpu().numpy().view(np.uint32)


def _sort_cpu(keys, vals):
    o = np.argsort(keys, kind="stable")
    return keys[o], vals[o]


@pytest.mark.parametrize("n,num_cells", [
    (2, 8), (3, 64), (255, 256), (256, 256), (257, 2 ** 18), (4095, 2 ** 18), (4096, 2 ** 18),
    (4097, 2 ** 18), (100_000, 2 ** 24), (1_000_003, 2 ** 24), (300_000, 2 ** 12),
    (70_000, 2 ** 30), (50_000, 2 ** 32 - 1)])
def test_random_keys(n, num_cells):
    rng = np.random.default_rng(n)
    keys = rng.integers(0, num_cells, n, dtype=np.uint64).astype(np.uint32)
    vals = rng.permutation(n).astype(np.uint32)
    k, v = _sort_gpu(keys, vals, num_cells)
    rk, rv = _sort_cpu(keys, vals)
    np.testing.assert_array_equal(k, rk)
    np.testing.assert_array_equal(v, rv)


@pytest.mark.parametrize("pattern", ["equal", "sorted", "reversed", "few", "blocks"])
def test_key_patterns(pattern):
    n, cells = 200_000, 2 ** 18
    rng = np.random.default_rng(5)
    if pattern == "equal":
        keys = np.full(n, 12345, np.uint32)
    elif pattern == "sorted":
        keys = np.sort(rng.integers(0, cells, n)).astype(np.uint32)
    elif pattern == "reversed":
        keys = np.sort(rng.integers(0, cells, n))[::-1].astype(np.uint32).copy()
    elif pattern == "few":
        keys = rng.choice(np.array([0, 7, 1 << 17, cells - 1], np.uint32), n)
    else:  # runs of identical keys, as cells of a sorted particle array
        keys = np.repeat(rng.integers(0, cells, n // 50), 50).astype(np.uint32)
    vals = np.arange(n, dtype=np.uint32)
    k, v = _sort_gpu(keys, vals, cells)
    rk, rv = _sort_cpu(keys, vals)
    np.testing.assert_array_equal(k, rk)
    np.testing.assert_array_equal(v, rv)


def test_key_above_grid_is_reported():
    from fullc0ntact_gb300 import _native
    keys = np.arange(1000, dtype=np.uint32)
    keys[500] = 1 << 20
    with pytest.raises(_native.FcdemError, match="key width"):
        _sort_gpu(keys, np.arange(1000, dtype=np.uint32), 4096)


def test_repeated_sorts_reuse_scratch():
    rng = np.random.default_rng(9)
    for n in [10_000, 500_000, 20_000, 500_000]:
        keys = rng.integers(0, 2 ** 24, n).astype(np.uint32)
        vals = np.arange(n, dtype=np.uint32)
        k, v = _sort_gpu(keys, vals, 2 ** 24)
        rk, rv = _sort_cpu(keys, vals)
        np.testing.assert_array_equal(v, rv)


@pytest.mark.parametrize("n", [5000, 300_001])
def test_every_pass_configuration_sorts_identically(n):
    from fullc0ntact_gb300 import dem
    lib = dem.lib
    count = lib.fcdemSetSortConfig(n, -1)
    assert count >= 2
    rng = np.random.default_rng(n + 1)
    keys = rng.integers(0, 2 ** 24, n).astype(np.uint32)
    vals = np.arange(n, dtype=np.uint32)
    rk, rv = _sort_cpu(keys, vals)
    try:
        for k in range(count):
            assert lib.fcdemSetSortConfig(n, k) == count
            gk, gv = _sort_gpu(keys, vals, 2 ** 24)
            np.testing.assert_array_equal(gk, rk)
            np.testing.assert_array_equal(gv, rv)
    finally:
        lib.fcdemSetSortConfig(n, -1)


def test_autotune_picks_a_configuration():
    import ctypes as C
    from fullc0ntact_gb300 import dem
    t = C.c_float()
    best = dem.lib.fcdemAutotuneSort(200_000, 2 ** 24, C.byref(t))
    dem.check("autotune")
    assert best >= 0 and t.value > 0.0
    keys = np.random.default_rng(3).integers(0, 2 ** 24, 200_000).astype(np.uint32)
    vals = np.arange(200_000, dtype=np.uint32)
    gk, gv = _sort_gpu(keys, vals, 2 ** 24)
    rk, rv = _sort_cpu(keys, vals)
    np.testing.assert_array_equal(gv, rv)
    dem.lib.fcdemSetSortConfig(200_000, -1)


def test_lookback_wait_that_runs_out_is_reported_and_recovers():
    """The look-back wait of the radix sort is bounded.  With a limit of zero
    rounds every tile after the first gives up at once: the sort records
    FCDEM_ERR_DEVICE_TIMEOUT, and its writes stay inside the arrays (a
    partial prefix is at most the true one; the guard words around the
    arrays are untouched).  With the default limit restored the next sort is
    correct."""
    from fullc0ntact_gb300 import dem
    from fullc0ntact_gb300.params import make_params
    lib = dem.lib
    n, cells, pad = 300_000, 2 ** 24, 4096  # 74 tiles of 4096 keys, 3 passes
    rng = np.random.default_rng(77)
    keys = rng.integers(0, cells, n).astype(np.uint32)
    vals = np.arange(n, dtype=np.uint32)
    P = make_params(n, (256, 256, 256), 0.01)
    dem.set_parameters(P)
    guard = -123456789
    kb = torch.full((n + 2 * pad,), guard, dtype=torch.int32, device="cuda")
    vb = torch.full((n + 2 * pad,), guard, dtype=torch.int32, device="cuda")
    kb[pad:pad + n] = torch.from_numpy(keys.view(np.int32)).cuda()
    vb[pad:pad + n] = torch.from_numpy(vals.view(np.int32)).cuda()
    assert lib.fcdemGetLastError() == 0
    try:
        lib.fcdemSetSortWaitLimit(0)
        lib.sortParticles(kb.data_ptr() + 4 * pad, vb.data_ptr() + 4 * pad, n)
        code = lib.fcdemGetLastError()
    finally:
        lib.fcdemSetSortWaitLimit(-1)
    assert code == 5, code  # FCDEM_ERR_DEVICE_TIMEOUT
    for b in (kb, vb):
        assert bool((b[:pad] == guard).all()) and bool((b[pad + n:] == guard).all())
    k, v = _sort_gpu(keys, vals, cells)  # the context still works
    rk, rv = _sort_cpu(keys, vals)
    np.testing.assert_array_equal(k, rk)
    np.testing.assert_array_equal(v, rv)
