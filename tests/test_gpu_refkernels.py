"""The product kernels against the reference's OWN kernels compiled for
sm_103a (oracle/_ref/fcref_kernels.cubin, built from cuda_addon/
particles_kernel.cu by oracle/Makefile) on the same GPU and the same inputs.
Skipped where that cubin was not built."""
import numpy as np
import pytest
import torch

from fcdem_testutil import REL_TOL, force_floor, product_params, oracle_params, rel_err_vec

pytestmark = pytest.mark.gpu


def _ref():
    from oracle import oracle as O
    try:
        R = O.ref_gpu()
    except RuntimeError as e:  # present but not loadable: a real failure
        pytest.fail(str(e))
    if R is None:
        pytest.skip("oracle/_ref/fcref_kernels.cubin not built here")
    return R


def _run_ref(R, P, pos0, vel0, dt):
    import ctypes as C
    from oracle import oracle as O
    n, ncell = pos0.shape[0], P.numCells
    pos = torch.from_numpy(pos0.copy()).cuda()
    vel = torch.from_numpy(vel0.copy()).cuda()
    torch.cuda.synchronize()
    OP = oracle_params(bytes(P))
    assert R.fcrefgpu_set_parameters(C.byref(OP)) == 0
    assert R.fcrefgpu_integrate(pos.data_ptr(), vel.data_ptr(), dt, n, None) == 0
    h = torch.empty(n, dtype=torch.int32, device="cuda")
    x = torch.empty_like(h)
    assert R.fcrefgpu_calc_hash(h.data_ptr(), x.data_ptr(), pos.data_ptr(), n, None) == 0
    torch.cuda.synchronize()
    hash0 = h.clone()
    # thrust::sort_by_key on uint keys = stable ascending order (restated)
    hk = h.cpu().numpy().view(np.uint32)
    o = np.argsort(hk, kind="stable")
    hs = torch.from_numpy(hk[o].view(np.int32).copy()).cuda()
    xs = torch.from_numpy(x.cpu().numpy()[o].copy()).cuda()
    cs = torch.empty(ncell, dtype=torch.int32, device="cuda")
    ce = torch.full((ncell,), -1, dtype=torch.int32, device="cuda")
    sp, sv = torch.empty_like(pos), torch.empty_like(vel)
    assert R.fcrefgpu_reorder(cs.data_ptr(), ce.data_ptr(), sp.data_ptr(), sv.data_ptr(),
                              hs.data_ptr(), xs.data_ptr(), pos.data_ptr(), vel.data_ptr(),
                              n, ncell, None) == 0
    nv = vel.clone()
    assert R.fcrefgpu_collide(nv.data_ptr(), sp.data_ptr(), sv.data_ptr(), xs.data_ptr(),
                              cs.data_ptr(), ce.data_ptr(), n, None) == 0
    torch.cuda.synchronize()
    return dict(pos=pos.cpu().numpy(), vel=vel.cpu().numpy(), hash=hash0.cpu().numpy(),
                hash_sorted=hs.cpu().numpy(), index_sorted=xs.cpu().numpy(),
                cs=cs.cpu().numpy(), ce=ce.cpu().numpy(), sp=sp.cpu().numpy(),
                nv=nv.cpu().numpy())


@pytest.mark.parametrize("which", ["lattice", "random", "wrap"])
def test_product_matches_reference_kernels(which):
    from fullc0ntact_gb300 import dem, scenes
    R = _ref()
    if which == "lattice":
        sc = scenes.lattice_scene()
    elif which == "random":
        sc = scenes.random_box(20000, grid=(32, 32, 32), radius=1.0 / 32.0, seed=4)
    else:
        sc = scenes.random_box(3000, grid=(4, 4, 4), radius=0.07, cell=0.25, seed=5)
    ref = _run_ref(R, sc["params"], sc["pos"], sc["vel"], sc["dt"])
    ds = dem.DeviceScene(sc)
    ds.stages()
    dem.check()
    for k_ref, t in [("pos", ds.pos), ("vel", ds.vel)]:
        pass
    np.testing.assert_array_equal(ds.pos.cpu().numpy().view(np.uint32), ref["pos"].view(np.uint32))
    np.testing.assert_array_equal(ds.hash.cpu().numpy(), ref["hash_sorted"])
    np.testing.assert_array_equal(ds.index.cpu().numpy(), ref["index_sorted"])
    cs = ds.cell_start.cpu().numpy()
    np.testing.assert_array_equal(cs, ref["cs"])
    ne = cs != -1
    np.testing.assert_array_equal(ds.cell_end.cpu().numpy()[ne], ref["ce"][ne])
    np.testing.assert_array_equal(ds.sorted_pos.cpu().numpy(), ref["sp"])
    out = ds.vel.cpu().numpy()
    vin = ref["vel"]
    f_ref = ref["nv"][:, :3].astype(np.float64) - vin[:, :3]
    f_gpu = out[:, :3].astype(np.float64) - vin[:, :3]
    e = rel_err_vec(f_gpu, f_ref, force_floor(f_ref))
    bitexact = np.mean(np.all(out.view(np.uint32) == ref["nv"].view(np.uint32), axis=1))
    print(f"{which}: force rel err max {e.max():.3e}; bit-identical rows {bitexact:.6f}")
    assert e.max() <= REL_TOL
