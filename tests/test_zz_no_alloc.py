"""fcdemSortParticlesNoAlloc: the sort for callers that must not have the
library allocate device memory (graph capture, host-owned memory pools,
runs at the memory limit).  It must give exactly what sortParticles gives,
on two calls in a row, without allocating, and refuse sizes above its fixed
scratch.  This file is collected last so that a failure here cannot hide the
results of the other tests."""
import ctypes as C

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
