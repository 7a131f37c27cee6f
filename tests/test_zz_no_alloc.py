"""fcdemSortParticlesNoAlloc: the sort for callers that must not have the
library allocate device memory (hosts whose own pool owns every byte of
device memory, runs at the memory limit).  It must give exactly what
sortParticles gives, on two calls in a row, without allocating, on every
pass route (1, 2, 3 and 4 radix passes), report a look-back wait that ran
out through fcdemGetLastError, and refuse sizes above its fixed scratch.
This file is collected last so that a failure here cannot hide the results
of the other tests."""
import os
import subprocess
import sys

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

MAX_PARTICLES = 1 << 20


def _keys(rng, n, num_cells):
    keys = rng.integers(0, num_cells, n, dtype=np.uint64).astype(np.uint32)
    vals = rng.permutation(n).astype(np.uint32)
    return (torch.from_numpy(keys.view(np.int32)).cuda(),
            torch.from_numpy(vals.view(np.int32)).cuda())


def test_no_alloc_sort_matches_sort_particles():
    from fullc0ntact_gb300 import dem
    from fullc0ntact_gb300.params import make_params
    lib = dem.lib
    P = make_params(MAX_PARTICLES, (256, 256, 256), 1.0 / 256.0)
    dem.set_parameters(P)
    rng = np.random.default_rng(20261203)
    cases = [(MAX_PARTICLES, 256 ** 3), (300_001, 256 ** 3)]
    inputs = [_keys(rng, n, c) for n, c in cases]
    expect = []
    for k, v in inputs:  # the allocating sort first (also loads the module)
        k2, v2 = k.clone(), v.clone()
        lib.sortParticles(k2.data_ptr(), v2.data_ptr(), k2.numel())
        expect.append((k2, v2))
    torch.cuda.synchronize()
    dem.check("sortParticles")
    outs = []
    for k, v in inputs:  # two calls in a row sharing the static scratch
        k3, v3 = k.clone(), v.clone()
        outs.append((k3, v3))
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    for k3, v3 in outs:
        lib.fcdemSortParticlesNoAlloc(k3.data_ptr(), v3.data_ptr(), k3.numel())
    torch.cuda.synchronize()
    free_after = torch.cuda.mem_get_info()[0]
    dem.check("fcdemSortParticlesNoAlloc")
    assert free_after == free_before, "the no-alloc sort changed free device memory"
    for (k2, v2), (k3, v3) in zip(expect, outs):
        assert torch.equal(k2, k3)
        assert torch.equal(v2, v3)


def test_no_alloc_sort_refuses_oversize():
    from fullc0ntact_gb300 import dem
    lib = dem.lib
    n = MAX_PARTICLES + 1
    k = torch.arange(n, 0, -1, dtype=torch.int32, device="cuda")
    v = torch.arange(n, dtype=torch.int32, device="cuda")
    k0, v0 = k.clone(), v.clone()
    lib.fcdemSortParticlesNoAlloc(k.data_ptr(), v.data_ptr(), n)
    assert lib.fcdemGetLastError() == 1  # FCDEM_ERR_INVALID_VALUE
    assert torch.equal(k, k0) and torch.equal(v, v0)


@pytest.mark.parametrize("num_cells", [200, 1 << 16])
def test_no_alloc_sort_one_and_two_passes(num_cells):
    """numCells <= 256: one pass (result copied back from the scratch);
    2^16: two passes (A -> B -> A)."""
    from fullc0ntact_gb300 import dem
    from fullc0ntact_gb300.params import make_params
    lib = dem.lib
    P = make_params(100_000, (8, 8, 4), 0.01)
    P.numCells = num_cells
    dem.set_parameters(P)
    rng = np.random.default_rng(num_cells)
    for n in (100_000, 4097):
        k, v = _keys(rng, n, num_cells)
        k2, v2 = k.clone(), v.clone()
        lib.sortParticles(k2.data_ptr(), v2.data_ptr(), n)
        lib.fcdemSortParticlesNoAlloc(k.data_ptr(), v.data_ptr(), n)
        dem.check("sorts")
        assert torch.equal(k, k2) and torch.equal(v, v2)


def test_no_alloc_sort_reports_a_wait_that_ran_out():
    """The sort's status word lives in its static scratch; a look-back wait
    that runs out (limit of zero rounds) reaches fcdemGetLastError, and the
    next call with the default limit is correct."""
    from fullc0ntact_gb300 import dem
    from fullc0ntact_gb300.params import make_params
    lib = dem.lib
    dem.set_parameters(make_params(300_000, (256, 256, 256), 0.01))
    rng = np.random.default_rng(31)
    k, v = _keys(rng, 300_000, 1 << 24)
    k0, v0 = k.clone(), v.clone()
    assert lib.fcdemGetLastError() == 0
    try:
        lib.fcdemSetSortWaitLimit(0)
        lib.fcdemSortParticlesNoAlloc(k.data_ptr(), v.data_ptr(), k.numel())
        code = lib.fcdemGetLastError()
    finally:
        lib.fcdemSetSortWaitLimit(-1)
    assert code == 5, code  # FCDEM_ERR_DEVICE_TIMEOUT
    k.copy_(k0)
    v.copy_(v0)
    lib.fcdemSortParticlesNoAlloc(k.data_ptr(), v.data_ptr(), k.numel())
    lib.sortParticles(k0.data_ptr(), v0.data_ptr(), k0.numel())
    dem.check("after the timeout")
    assert torch.equal(k, k0) and torch.equal(v, v0)


_FRESH = r"""
import sys
import numpy as np
import torch
sys.path.insert(0, sys.argv[1])
from fullc0ntact_gb300 import dem
n = 200_003
rng = np.random.default_rng(5)
keys = rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32)
vals = rng.permutation(n).astype(np.uint32)
k = torch.from_numpy(keys.view(np.int32)).cuda()
v = torch.from_numpy(vals.view(np.int32)).cuda()
dem.lib.fcdemSortParticlesNoAlloc(k.data_ptr(), v.data_ptr(), n)  # no setParameters yet
dem.check("no-alloc sort")
o = np.argsort(keys, kind="stable")
assert np.array_equal(k.cpu().numpy().view(np.uint32), keys[o])
assert np.array_equal(v.cpu().numpy().view(np.uint32), vals[o])
print("ok")
"""


def test_no_alloc_sort_before_set_parameters_sorts_32_bit_keys():
    """In a fresh process with no setParameters call the key width is 32
    bits (four passes, A -> B -> A -> B -> A); checked against numpy's
    stable sort."""
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, "-c", _FRESH, root], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0 and "ok" in r.stdout, r.stdout + r.stderr
