"""Whole runs of the packed polydisperse scene (4,194,304 lognormal spheres
in a 256^3 grid, 500 steps, and a 100,000-sphere version of it):

* the hashes, the permutation and the cell ranges of every step of the full
  500-step job through fcdemUpdate equal, bit for bit, those of the
  reference-named staged calls (integrateSystem, calcHash, sortParticles --
  an independent radix sort -- reorderDataAndFindCellStart, collide) from the
  same state; the staged calls are pinned to the oracle on the same kind of
  scene in test_gpu_stages.py and test_gpu_collide_paths.py;
* one 500-step fcdemUpdate call (the state kept in sorted order between
  steps) ends in exactly the state of 500 single-step calls;
* trajectories are chaotic, so a 100-step run is compared with the oracle's
  (host arithmetic, every product rounded) by total kinetic and potential
  energy, momentum and contact count, and with the oracle in the GPU's
  fused arithmetic, whose run has the same statistics exactly; the same
  comparison by statistics for 60 steps of the unified-memory step
  (evalForces, integrate with the torus distance map, the cylinder and the
  planes) of the torus fall."""
import numpy as np
import pytest
import torch

from fcdem_testutil import oracle_params

pytestmark = pytest.mark.gpu


def _bits(t: torch.Tensor) -> torch.Tensor:
    return t.view(torch.int32)  # NaN-safe bitwise comparison of float tensors


def test_packed_job_tables_bit_exact_every_step():
    from fullc0ntact_gb300 import dem, scenes
    sc = scenes.packed_scene(4_194_304)
    a, b, c = dem.DeviceScene(sc), dem.DeviceScene(sc), dem.DeviceScene(sc)
    steps = 500
    for k in range(steps):
        b.pos.copy_(a.pos)
        b.vel.copy_(a.vel)
        a.update(1)
        b.stages()
        assert torch.equal(a.hash, b.hash), k
        assert torch.equal(a.index, b.index), k
        assert torch.equal(a.cell_start, b.cell_start), k
        occupied = a.cell_start != -1
        assert torch.equal(a.cell_end[occupied], b.cell_end[occupied]), k
        assert torch.equal(_bits(a.pos), _bits(b.pos)), k
        assert torch.equal(_bits(a.vel), _bits(b.vel)), k
    dem.check("500 single steps")
    c.update(steps)
    dem.check("one 500-step call")
    assert torch.equal(_bits(a.pos), _bits(c.pos))
    assert torch.equal(_bits(a.vel), _bits(c.vel))
    assert torch.equal(a.hash, c.hash) and torch.equal(a.index, c.index)
    # the job reaches its late state: particles with NaN coordinates
    # (coincident equal spheres in a box corner) and crowded cells
    nan = int(torch.isnan(a.pos[:, :3]).any(dim=1).sum())
    print(f"after {steps} steps: {nan} particles with a NaN coordinate")
    assert nan > 0


def _stats(pos, vel, params, radius_from_w, with_collider=True):
    from oracle import oracle as O
    v = vel[:, :3].astype(np.float64)
    ok = np.isfinite(pos[:, :3]).all(axis=1) & np.isfinite(v).all(axis=1)
    ke = 0.5 * np.sum(v[ok] ** 2)
    pe = -params.gravity[2] * np.sum(pos[ok, 2].astype(np.float64) + 1.0)
    mom = v[ok].sum(axis=0)
    h, x = O.calc_hash(params, pos)
    hs, xs = O.sort_pairs(h, x)
    cs, ce, sp, sv = O.reorder(hs, xs, pos, vel, params.numCells)
    nv = O.collide(params, sp, sv, xs, cs, ce, radius_from_w, with_collider)
    contacts = int(np.count_nonzero(np.any(nv[:, :3] != vel[:, :3], axis=1)))
    return ke, pe, mom, contacts


def test_packed_multistep_statistics_match_oracle():
    from fullc0ntact_gb300 import dem, scenes
    from oracle import oracle as O
    sc = scenes.packed_scene(100_000, grid=128)
    steps = 100
    ds = dem.DeviceScene(sc)
    ds.update(steps)
    dem.check("update")
    P = oracle_params(bytes(sc["params"]))
    pos, vel = sc["pos"].copy(), sc["vel"].copy()
    O.update(P, pos, vel, sc["dt"], steps=steps, radius_from_w=True)
    g = _stats(ds.pos.cpu().numpy(), ds.vel.cpu().numpy(), P, True)
    o = _stats(pos, vel, P, True)
    print(f"GPU ke {g[0]:.6e} pe {g[1]:.6e} contacts {g[3]}; "
          f"oracle ke {o[0]:.6e} pe {o[1]:.6e} contacts {o[3]}")
    # the host arithmetic rounds every product, the GPU fuses them: over 100
    # steps of the hot packing the trajectories part (chaos), and the
    # contact count, a count of near-threshold pairs, moves by a few percent
    assert abs(g[0] - o[0]) <= 0.02 * o[0]
    assert abs(g[1] - o[1]) <= 1e-3 * abs(o[1])
    assert np.all(np.abs(g[2] - o[2]) <= 0.05 * np.abs(o[2]).max() + 1e-9)
    assert abs(g[3] - o[3]) <= 0.04 * o[3]
    # with the GPU's fused arithmetic the oracle's run has the same statistics
    pos, vel = sc["pos"].copy(), sc["vel"].copy()
    with O.gpu_arithmetic():
        O.update(P, pos, vel, sc["dt"], steps=steps, radius_from_w=True)
    f = _stats(pos, vel, P, True)
    assert f[0] == g[0] and f[1] == g[1] and f[3] == g[3]


def test_um_torus_fall_statistics_match_oracle():
    from fullc0ntact_gb300 import dem, scenes
    from oracle import oracle as O
    sc = scenes.torus_fall_scene(100_000, z0=0.09)  # the lowest layers start at the torus
    dmap = dem.DistanceMap.torus(0.3, 0.1, 128, 0.05)
    steps = 60
    ds = dem.UmScene(sc, dmap)
    ds.update(steps)
    dem.check("um update")
    P = oracle_params(bytes(sc["params"]))
    w = bool(sc.get("radius_from_w", False))
    v = dmap.vertices()
    m = O.distmap_struct(dmap.vmin, dmap.vmax, dmap.cell_size, dmap.cells,
                         np.ascontiguousarray(v[:, 0]), np.ascontiguousarray(v[:, 1:]))
    pos, vel = sc["pos"].copy(), sc["vel"].copy()
    for _ in range(steps):  # calcHash, sortParticles, reorder, evalForces, integrateSystem
        h, x = O.calc_hash(P, pos)
        hs, xs = O.sort_pairs(h, x)
        cs, ce, sp, sv = O.reorder(hs, xs, pos, vel, P.numCells)
        vel = O.collide(P, sp, sv, xs, cs, ce, w, False)
        O.integrate_distmap(P, m, pos, vel, sc["dt"], w)
    g = _stats(ds.pos.cpu().numpy(), ds.vel.cpu().numpy(), P, w, False)
    o = _stats(pos, vel, P, w, False)
    print(f"GPU ke {g[0]:.6e} pe {g[1]:.6e} contacts {g[3]}; "
          f"oracle ke {o[0]:.6e} pe {o[1]:.6e} contacts {o[3]}")
    assert o[3] > 1000  # the spheres are on the torus and on each other
    assert abs(g[0] - o[0]) <= 0.02 * o[0]
    assert abs(g[1] - o[1]) <= 1e-3 * abs(o[1])
    assert np.all(np.abs(g[2] - o[2]) <= 0.05 * np.abs(o[2]).max() + 1e-9)
    assert abs(g[3] - o[3]) <= 0.02 * o[3]
