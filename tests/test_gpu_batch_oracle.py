"""Batched scenes against the oracle, scene by scene.

Each scene of a batch is one ParticleSystem with its own parameters and its
own box.  The oracle steps it alone (oracle.batch_scene_step: the integrate
in the scene's box -- with the obstacle's checkDistMap in the obstacle
batches -- calcHash, sortParticles, reorder, collide), with the GPU's fused
arithmetic (oracle.gpu_arithmetic).  Single steps are compared on the same
input state:

* the integrated positions bit for bit in box batches; in obstacle batches
  within 2e-7 (the GPU normalises the contact normal with rsqrtf, within 2
  ulp of the oracle's 1/sqrtf);
* the collide on the same input (the batch's own positions, the oracle's
  integrated velocities): the new velocities bit for bit; the force error
  of the oracle's host arithmetic (every product rounded) is printed.

A 100-step run of the box batch ends in the oracle's bits.  Obstacle
batches drift apart by the rsqrtf roundings and are chaotic, so a 100-step
run is compared by total kinetic and potential energy, momentum and contact
count."""
import numpy as np
import pytest
import torch

from fcdem_testutil import REL_TOL, assert_same_floats, force_floor, rel_err_vec

pytestmark = pytest.mark.gpu

POS_TOL_OBSTACLE = 2e-7


def _box_batch(num=12, seed=5, big=True):
    from fullc0ntact_gb300 import scenes
    rng = np.random.default_rng(seed)
    sizes = list(np.exp(rng.uniform(np.log(1024), np.log(8000), num)).astype(int))
    if big:
        sizes[num // 2] = 65_536  # the largest scene of the batched workload
    return [scenes.batch_scene(int(n), 1000 + k) for k, n in enumerate(sizes)]


def _obstacle_batch(num=6, seed=5):
    from fullc0ntact_gb300 import scenes
    return scenes.batch_obstacle_scenes(num, 3000, 20000, seed=seed, num_shapes=4)


def _oracle_maps(maps):
    from oracle import oracle as O
    out = []
    for m in maps:
        v = m.vertices()
        out.append(O.distmap_struct(m.vmin, m.vmax, m.cell_size, m.cells,
                                    np.ascontiguousarray(v[:, 0]),
                                    np.ascontiguousarray(v[:, 1:])))
    return out


def _compare_step(b, scs, host_pos, host_vel, omaps=None, shape=None):
    """b has just made one update from (host_pos, host_vel); compare every
    scene with the oracle.  Returns (max force error, map contacts)."""
    from oracle import oracle as O
    pos_g = b.split(b.pos)
    vel_g = b.split(b.vel)
    starts = np.cumsum([0] + b.sizes)
    worst, contacts, pos_err = 0.0, 0, 0.0
    for k, sc in enumerate(scs):
        a, e = starts[k], starts[k + 1]
        p_in, v_in = host_pos[a:e].copy(), host_vel[a:e].copy()
        obstacle = omaps is not None
        m = omaps[shape[k]] if obstacle and shape[k] >= 0 else None
        P = O.SimParams.from_buffer_copy(bytes(sc["params"]))
        w = bool(sc.get("radius_from_w", False))
        lo, hi = O._box(sc)
        po, vo = p_in.copy(), v_in.copy()
        with O.gpu_arithmetic():
            if obstacle:
                contacts += O.batch_obstacle_integrate(P, lo, hi, m, po, vo, sc["dt"], w)
            else:
                O.integrate_box(P, lo, hi, po, vo, sc["dt"], w)
        pg = pos_g[k].cpu().numpy()
        vg = vel_g[k].cpu().numpy()
        if obstacle:
            np.testing.assert_allclose(pg[:, :3], po[:, :3], rtol=0, atol=POS_TOL_OBSTACLE)
            pos_err = max(pos_err, float(np.abs(pg[:, :3] - po[:, :3]).max()))
        else:
            np.testing.assert_array_equal(pg.view(np.uint32), po.view(np.uint32))
        # the collide on the same input: the batch's positions, the oracle's velocities
        h, x = O.calc_hash(P, pg)
        hs, xs = O.sort_pairs(h, x)
        cs, ce, sp, sv = O.reorder(hs, xs, pg, vo, P.numCells)
        with O.gpu_arithmetic():
            nv = O.collide(P, sp, sv, xs, cs, ce, w, True)
        assert_same_floats(vg[:, :3], nv[:, :3])
        nv_host = O.collide(P, sp, sv, xs, cs, ce, w, True)
        f_ref = nv_host[:, :3].astype(np.float64) - vo[:, :3]
        f_gpu = vg[:, :3].astype(np.float64) - vo[:, :3]
        err = rel_err_vec(f_gpu, f_ref, force_floor(f_ref))
        assert err.max() <= REL_TOL, (k, float(err.max()))
        worst = max(worst, float(err.max()))
    if obstacle:
        print(f"obstacle integrate: max position difference {pos_err:.2e}")
    return worst, contacts


@pytest.mark.parametrize("graph", [False, True])
def test_box_batch_single_steps_match_oracle(graph):
    """Batched plain DEM (non-unit boxes, per-scene grids): three single
    steps, each from the batch's own state, against the oracle per scene."""
    from fullc0ntact_gb300 import dem
    scs = _box_batch()
    b = dem.Batch(scs)
    worst = 0.0
    for step in range(3):
        hp, hv = b.pos.cpu().numpy().copy(), b.vel.cpu().numpy().copy()
        b.update(1, graph=graph)
        dem.check("batch step")
        e, _ = _compare_step(b, scs, hp, hv)
        worst = max(worst, e)
    print(f"box batch: bit-exact; force error of the host arithmetic {worst:.2e}")


def test_box_batch_multistep_call_equals_single_steps():
    """One 6-step call (the next integrate fused into each collide, the state
    kept in slot order) ends in the bits of six single-step calls, which the
    previous test pins to the oracle."""
    from fullc0ntact_gb300 import dem
    scs = _box_batch(8, seed=7, big=False)
    a, b = dem.Batch(scs), dem.Batch(scs)
    a.update(6, graph=True)
    for _ in range(6):
        b.update(1, graph=False)
    dem.check()
    assert torch.equal(a.pos.view(torch.int32), b.pos.view(torch.int32))
    assert torch.equal(a.vel.view(torch.int32), b.vel.view(torch.int32))


@pytest.mark.parametrize("neural", [False, True])
def test_obstacle_batch_single_steps_match_oracle(neural):
    """Batched DEM with obstacles (rounded boxes and tori, one map per
    scene): after 30 steps the spheres lie on their obstacles; two single
    steps from there against the oracle, with exact map queries and with the
    shape-conditioned network culling them."""
    from fullc0ntact_gb300 import dem, sdf
    scs, obs, shape = _obstacle_batch()
    maps = sdf.obstacle_maps(obs, 64)
    b = dem.Batch(scs)
    if neural:
        net, _ = sdf.shape_net(maps, samples_per_map=200_000, epochs=15)
        skin, _ = sdf.calibrate_skin(net, maps, 1.0 / 256.0, samples_per_map=200_000)
        b.set_obstacles(maps, shape, net=net, skin=skin)
    else:
        b.set_obstacles(maps, shape)
    b.update(30, graph=True)
    dem.check("advance")
    omaps = _oracle_maps(maps)
    worst, contacts = 0.0, 0
    for step in range(2):
        hp, hv = b.pos.cpu().numpy().copy(), b.vel.cpu().numpy().copy()
        b.update(1, graph=False)
        dem.check("obstacle batch step")
        e, c = _compare_step(b, scs, hp, hv, omaps, shape)
        worst, contacts = max(worst, e), contacts + c
    print(f"obstacle batch (neural={neural}): velocities bit-exact, force error of the host "
          f"arithmetic {worst:.2e}, {contacts} map contacts")
    assert contacts > 100  # the spheres are on their obstacles


def _stats(scs, pos, vel):
    """Total kinetic and potential energy, momentum and contact count of a
    list of scene states (contacts: particles whose collide changes their
    velocity, by the oracle)."""
    from oracle import oracle as O
    ke = pe = 0.0
    mom = np.zeros(3)
    contacts = 0
    for sc, p, v in zip(scs, pos, vel):
        P = O.SimParams.from_buffer_copy(bytes(sc["params"]))
        w = bool(sc.get("radius_from_w", False))
        v3 = v[:, :3].astype(np.float64)
        ok = np.isfinite(p[:, :3]).all(axis=1) & np.isfinite(v3).all(axis=1)
        ke += 0.5 * np.sum(v3[ok] ** 2)
        pe += -P.gravity[2] * np.sum(p[ok, 2].astype(np.float64) - float(sc["box_lo"][2]))
        mom += v3[ok].sum(axis=0)
        h, x = O.calc_hash(P, p)
        hs, xs = O.sort_pairs(h, x)
        cs, ce, sp, sv = O.reorder(hs, xs, p, v, P.numCells)
        nv = O.collide(P, sp, sv, xs, cs, ce, w, True)
        contacts += int(np.count_nonzero(np.any(nv[:, :3] != v[:, :3], axis=1)))
    return ke, pe, mom, contacts


@pytest.mark.parametrize("kind", ["box", "obstacle"])
def test_batch_multistep_statistics_match_oracle(kind):
    from fullc0ntact_gb300 import dem, sdf
    from oracle import oracle as O
    steps = 100
    if kind == "box":
        scs = _box_batch(10, seed=11, big=False)
        shape, omaps = None, None
        b = dem.Batch(scs)
    else:
        scs, obs, shape = _obstacle_batch(6, seed=8)
        maps = sdf.obstacle_maps(obs, 64)
        omaps = _oracle_maps(maps)
        b = dem.Batch(scs)
        b.set_obstacles(maps, shape)
    b.update(steps, graph=True)
    dem.check("batch run")
    gpos = [t.cpu().numpy() for t in b.split(b.pos)]
    gvel = [t.cpu().numpy() for t in b.split(b.vel)]
    opos, ovel = [], []
    with O.gpu_arithmetic():
        for k, sc in enumerate(scs):
            p, v = sc["pos"].copy(), sc["vel"].copy()
            m = omaps[shape[k]] if omaps is not None else None
            for _ in range(steps):
                st = O.batch_scene_step(sc, m, obstacle=omaps is not None, pos=p, vel=v)
                p, v = st["pos"], st["newVel"]
            opos.append(p)
            ovel.append(v)
    if kind == "box":  # the same arithmetic throughout: the same bits
        for k in range(len(scs)):
            assert_same_floats(gpos[k], opos[k])
            assert_same_floats(gvel[k][:, :3], ovel[k][:, :3])
    g = _stats(scs, gpos, gvel)
    o = _stats(scs, opos, ovel)
    print(f"{kind}: GPU ke {g[0]:.6e} pe {g[1]:.6e} contacts {g[3]}; "
          f"oracle ke {o[0]:.6e} pe {o[1]:.6e} contacts {o[3]}")
    assert o[3] > 1000
    assert abs(g[0] - o[0]) <= 0.02 * o[0]
    assert abs(g[1] - o[1]) <= 1e-3 * abs(o[1])
    assert np.all(np.abs(g[2] - o[2]) <= 0.05 * np.abs(o[2]).max() + 1e-9)
    assert abs(g[3] - o[3]) <= 0.02 * o[3]
