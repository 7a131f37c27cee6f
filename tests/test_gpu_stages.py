"""The CUDA stages through the C-ABI against the reference's golden fixtures
and the CPU oracle: hash, sort, cell ranges and reorder bit for bit, collide
within the 1e-5 relative bar."""
import numpy as np
import pytest
import torch

from fcdem_testutil import (GOLDEN_CASES, REL_TOL, check_cell_tables, force_floor,
                            full_cells, load_golden, oracle_params, product_params,
                            rel_err_vec)

pytestmark = pytest.mark.gpu


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _i32(a):
    return torch.from_numpy(np.ascontiguousarray(a).view(np.int32)).cuda()


def _u32(t):
    return t.cpu().numpy().view(np.uint32)


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_stages_match_reference_fixture(name):
    from fullc0ntact_gb300 import dem
    g = load_golden(name)
    P = product_params(g["params"])
    n, C = g["pos0"].shape[0], P.numCells
    dem.set_parameters(P)
    dem.set_radius_mode(False)
    pos, vel = _dev(g["pos0"]), _dev(g["vel0"])
    dem.integrate_system(pos, vel, float(g["dt"]), n)
    h = torch.empty(n, dtype=torch.int32, device="cuda")
    x = torch.empty_like(h)
    dem.calc_hash(h, x, pos, n)
    torch.cuda.synchronize()
    hash0, index0 = _u32(h), _u32(x)
    dem.sort_particles(h, x, n)
    cs = torch.empty(C, dtype=torch.int32, device="cuda")
    ce = torch.full((C,), -1, dtype=torch.int32, device="cuda")
    sp, sv = torch.empty_like(pos), torch.empty_like(vel)
    dem.reorder_data_and_find_cell_start(cs, ce, sp, sv, h, x, pos, vel, n, C)
    nv = vel.clone()
    dem.collide(nv, sp, sv, x, cs, ce, n, C)
    dem.check(name)

    # integrate and the hashing stages: bit-exact
    np.testing.assert_array_equal(pos.cpu().numpy().view(np.uint32), g["pos"].view(np.uint32))
    np.testing.assert_array_equal(vel.cpu().numpy().view(np.uint32), g["vel"].view(np.uint32))
    np.testing.assert_array_equal(hash0, g["hash"])
    np.testing.assert_array_equal(index0, g["index"])
    np.testing.assert_array_equal(_u32(h), g["hash_sorted"])
    np.testing.assert_array_equal(_u32(x), g["index_sorted"])
    ref_cs = full_cells(g, C)
    ce_full = _u32(ce)
    np.testing.assert_array_equal(_u32(cs), ref_cs)
    np.testing.assert_array_equal(ce_full[g["cells"]], g["cell_end"])
    np.testing.assert_array_equal(sp.cpu().numpy(), g["pos"][g["index_sorted"]])
    np.testing.assert_array_equal(sv.cpu().numpy(), g["vel"][g["index_sorted"]])
    # collide: the 1e-5 bar on the new velocity and on the force
    out = nv.cpu().numpy()
    assert np.all(out[:, 3] == 0.0)
    f_ref = g["new_vel"][:, :3].astype(np.float64) - g["vel"][:, :3]
    f_gpu = out[:, :3].astype(np.float64) - g["vel"][:, :3]
    e_v = rel_err_vec(out, g["new_vel"], 1e-6)
    e_f = rel_err_vec(f_gpu, f_ref, force_floor(f_ref))
    assert e_v.max() <= REL_TOL, e_v.max()
    assert e_f.max() <= REL_TOL, e_f.max()


@pytest.mark.parametrize("poly", [False, True])
def test_collide_matches_oracle_random(poly):
    """Polydisperse scenes (radius in pos.w) have no reference kernel: the
    oracle's restatement is the judge."""
    from fullc0ntact_gb300 import dem, scenes
    from oracle import oracle as O
    sc = scenes.random_box(6000, grid=(32, 32, 32), radius=1.0 / 24.0, seed=11, poly=poly)
    ds = dem.DeviceScene(sc)
    ds.stages()
    dem.check("stages")
    P = oracle_params(bytes(sc["params"]))
    st = O.step_stages(P, sc["pos"], sc["vel"], sc["dt"], radius_from_w=poly)
    np.testing.assert_array_equal(_u32(ds.hash), st["hash_sorted"])
    np.testing.assert_array_equal(_u32(ds.index), st["index_sorted"])
    check_cell_tables(_u32(ds.cell_start), _u32(ds.cell_end), st["cellStart"], st["cellEnd"])
    out = ds.vel.cpu().numpy()
    f_ref = st["newVel"][:, :3].astype(np.float64) - st["vel_in"][:, :3]
    f_gpu = out[:, :3].astype(np.float64) - st["vel_in"][:, :3]
    assert rel_err_vec(out, st["newVel"], 1e-6).max() <= REL_TOL
    assert rel_err_vec(f_gpu, f_ref, force_floor(f_ref)).max() <= REL_TOL


def test_error_against_fp64_oracle_is_small():
    """States the FP32 error against the FP64 evaluation of the same step."""
    from fullc0ntact_gb300 import dem
    from oracle import oracle as O
    g = load_golden("plain16k")
    Pp = product_params(g["params"])
    P = oracle_params(g["params"])
    ds = dem.DeviceScene(dict(pos=g["pos0"], vel=g["vel0"], params=Pp, dt=float(g["dt"])))
    ds.stages()
    dem.check()
    st = O.step_stages(P, g["pos0"], g["vel0"], float(g["dt"]))
    nv64 = O.collide_f64(P, st["sortedPos"], st["sortedVel"], st["index_sorted"],
                         st["cellStart"], st["cellEnd"])
    f64 = nv64[:, :3] - st["vel_in"][:, :3].astype(np.float64)
    f32 = ds.vel.cpu().numpy()[:, :3].astype(np.float64) - st["vel_in"][:, :3]
    err = rel_err_vec(f32, f64, force_floor(f64))
    print(f"plain16k force error vs FP64: max {err.max():.3e} median {np.median(err):.3e}")
    assert err.max() < 1e-4


def test_empty_and_tiny_inputs():
    from fullc0ntact_gb300 import dem
    from fullc0ntact_gb300.params import make_params
    P = make_params(0, (8, 8, 8), 0.1)
    dem.set_parameters(P)
    dem.set_radius_mode(False)
    z = torch.empty((0, 4), dtype=torch.float32, device="cuda")
    zi = torch.empty(0, dtype=torch.int32, device="cuda")
    cs = torch.empty(512, dtype=torch.int32, device="cuda")
    ce = torch.empty(512, dtype=torch.int32, device="cuda")
    # n = 0 through every stage: no work, no error
    dem.lib.integrateSystem(z.data_ptr() or None, z.data_ptr() or None, 0.5, 0)
    dem.lib.sortParticles(None, None, 0)
    dem.lib.reorderDataAndFindCellStart(cs.data_ptr(), ce.data_ptr(), None, None, None,
                                        None, None, None, 0, 512)
    dem.lib.collide(None, None, None, None, cs.data_ptr(), ce.data_ptr(), 0, 512)
    dem.check("n = 0")
    assert np.all(_u32(cs) == 0xFFFFFFFF)
    del zi


def test_errors_are_reported_not_fatal():
    from fullc0ntact_gb300 import dem, _native
    from fullc0ntact_gb300.params import make_params
    P = make_params(10, (6, 8, 8), 0.1)  # 6 is not a power of two
    dem.set_parameters(P)
    t = torch.zeros((10, 4), device="cuda")
    h = torch.zeros(10, dtype=torch.int32, device="cuda")
    dem.calc_hash(h, h.clone(), t, 10)
    with pytest.raises(_native.FcdemError):
        dem.check()
    dem.lib.registerGLBufferObject(1, None)
    assert dem.lib.fcdemGetLastError() == 4
    assert dem.lib.fcdemGetLastError() == 0


def test_tuning_and_culling_arguments_are_checked():
    """The tuning and culling entry points reject bad arguments with an error
    code and change nothing: a collide autotune of no particles, an unknown
    collide configuration, a negative Lipschitz bound or no network."""
    import ctypes as C
    from fullc0ntact_gb300 import dem, sdf  # sdf sets the culling calls' argument types
    lib = dem.lib
    lib.fcdemGetLastError()  # clear anything pending
    null = C.c_void_p()
    assert lib.fcdemAutotuneCollide(*([null] * 8), 0.5, 0, 8, None) == -1
    assert lib.fcdemGetLastError() == 1  # FCDEM_ERR_INVALID_VALUE
    lim = C.c_uint(7)
    assert lib.fcdemGetCollideConfig(30, C.byref(lim), None, None) == -1
    assert lim.value == 7 and lib.fcdemGetLastError() == 1
    assert lib.fcdemSetCollideConfig(-5) == 30  # out of range: the default
    lib.fcdemSdfSetTileCulling(None, 1.0)
    assert lib.fcdemGetLastError() == 1
    net = sdf.SdfNet(3, 64, 2, seed=1)
    lib.fcdemSdfSetTileCulling(net.handle, -1.0)
    assert lib.fcdemGetLastError() == 1
    net.set_tile_culling(0.0)
    assert lib.fcdemGetLastError() == 0
