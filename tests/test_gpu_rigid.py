"""Rigid particle clusters (d_integrateRigidBody, particledem_um.cu:640-718):
velocity and centre of mass under gravity and damping with only z stored,
member particles moved by v dt; the reference's two three-particle bodies
and general ones, against a numpy restatement."""
import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _fma32(a, b, c):
    return (np.float64(a) * np.float64(b) + np.float64(c)).astype(np.float32)


def test_rigid_bodies_match_restatement():
    from fullc0ntact_gb300 import dem
    from fullc0ntact_gb300.params import make_params
    rng = np.random.default_rng(4)
    n = 40
    pos = np.zeros((n, 4), np.float32)
    pos[:, :3] = rng.uniform(-0.5, 0.5, (n, 3))
    pos[:, 3] = rng.uniform(0.1, 0.9, n)
    specs = [(3, [0, 1, 2]), (3, [3, 4, 5]), (2, [10, 11, -1]), (1, [20, -1, -1]), (3, [30, 31, 39])]
    nb = len(specs)
    arr = (dem.RigidBody * nb)()
    for k, (m, idx) in enumerate(specs):
        arr[k].numParticles = m
        arr[k].indices[:] = idx
        arr[k].com[:] = list(rng.uniform(-0.3, 0.3, 3))
        arr[k].vel[:] = list(rng.uniform(-0.01, 0.01, 3))
    raw = np.frombuffer(bytes(arr), np.uint8).copy()
    g = (0.0, 0.0, -3e-4)
    dem.set_parameters(make_params(n, (16, 16, 16), 1.0 / 64.0, gravity=g, global_damping=0.99))
    d_bodies = torch.from_numpy(raw).cuda()
    d_pos = torch.from_numpy(pos.copy()).cuda()
    dt = np.float32(0.5)
    for _ in range(2):  # two calls in a row
        dem.um_integrate_rigid_bodies(d_bodies, nb, d_pos, n, float(dt))
    dem.check("rigid")
    out = dem.RigidBody * nb
    got = out.from_buffer_copy(d_bodies.cpu().numpy().tobytes())
    p_ref = pos.copy()
    ref = out.from_buffer_copy(bytes(arr))
    gr = np.array(g, np.float32)
    for _ in range(2):
        for k, (m, idx) in enumerate(specs):
            v = np.array(ref[k].vel[:], np.float32)
            v = _fma32(gr, dt, v)
            v = (v.astype(np.float64) * np.float64(np.float32(0.99))).astype(np.float32)
            ref[k].vel[2] = float(v[2])
            ref[k].com[2] = float(_fma32(v[2], dt, np.float32(ref[k].com[2])))
            for q in idx[:m]:
                if q >= 0:
                    p_ref[q, :3] = _fma32(v, dt, p_ref[q, :3])
                    p_ref[q, 3] = 1.0
    for k in range(nb):
        np.testing.assert_array_equal(np.array(got[k].com[:], np.float32),
                                      np.array(ref[k].com[:], np.float32))
        np.testing.assert_array_equal(np.array(got[k].vel[:], np.float32),
                                      np.array(ref[k].vel[:], np.float32))
    np.testing.assert_array_equal(d_pos.cpu().numpy(), p_ref)
