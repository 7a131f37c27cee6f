"""Neural signed-distance field of an obstacle (the C-ABI's fcdemSdf* calls).

``SdfNet`` wraps one network: FP32 master parameters on the device, trained
by the library's own forward/backward kernels and Adam on samples of a
``DistanceMap``; BF16 tensor-core inference; the culled boundary integrate
(``um_integrate_system_sdf``), whose results equal ``dem.um_integrate_system``
while the network's error stays below the skin band.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from ._native import check, lib
from .dem import DistanceMap, _p

vp = C.c_void_p
u32 = C.c_uint
f32 = C.c_float
_F3 = C.c_float * 3

_SIGS = {
    "fcdemSdfCreate": (vp, [C.c_int, C.c_int, C.c_int, C.c_ulonglong]),
    "fcdemSdfDestroy": (None, [vp]),
    "fcdemSdfNumParams": (u32, [vp]),
    "fcdemSdfGetParams": (None, [vp, vp]),
    "fcdemSdfSetParams": (None, [vp, vp]),
    "fcdemSdfSetNormalization": (None, [vp, _F3, _F3, f32]),
    "fcdemSdfGetNormalization": (None, [vp, _F3, _F3, C.POINTER(f32)]),
    "fcdemSdfSamples": (None, [vp, C.c_int, u32, f32, f32, C.c_ulonglong, vp, vp]),
    "fcdemSdfGradient": (f32, [vp, vp, vp, u32, f32, vp]),
    "fcdemSdfTrainSamples": (f32, [vp, vp, vp, u32, u32, u32, f32, f32]),
    "fcdemSdfEvalF32": (None, [vp, vp, vp, u32, vp]),
    "fcdemSdfInfer": (None, [vp, vp, vp, u32, vp]),
    "fcdemSdfSetTileCulling": (None, [vp, f32]),
    "fcdemUM_integrateSystemSdf": (None, [vp, vp, f32, u32, vp, vp, f32, vp]),
}
for _name, (_res, _args) in _SIGS.items():
    _f = getattr(lib, _name)
    _f.restype = _res
    _f.argtypes = _args


def _opt(t: torch.Tensor | None):
    return None if t is None else _p(t)


class SdfNet:
    """inputs = 3 + number of shape codes; hidden 64 or 128; 2 or 3 hidden
    layers (3 -> 64 -> 64 -> 64 -> 1 is SdfNet(3, 64, 3))."""

    def __init__(self, inputs: int = 3, hidden: int = 64, layers: int = 3, seed: int = 1):
        self.inputs, self.hidden, self.layers = inputs, hidden, layers
        h = lib.fcdemSdfCreate(inputs, hidden, layers, seed)
        check("fcdemSdfCreate")
        if not h:
            raise MemoryError("fcdemSdfCreate failed")
        self._h = h

    @property
    def handle(self):
        return self._h

    @property
    def num_params(self) -> int:
        return int(lib.fcdemSdfNumParams(self._h))

    def get_params(self) -> np.ndarray:
        out = np.zeros(self.num_params, np.float32)
        lib.fcdemSdfGetParams(self._h, out.ctypes.data)
        check("fcdemSdfGetParams")
        return out

    def set_params(self, p: np.ndarray) -> None:
        p = np.ascontiguousarray(p, np.float32)
        assert p.shape == (self.num_params,)
        lib.fcdemSdfSetParams(self._h, p.ctypes.data)
        check("fcdemSdfSetParams")

    def set_normalization(self, shift, scale, out_scale: float) -> None:
        lib.fcdemSdfSetNormalization(self._h, _F3(*map(float, shift)), _F3(*map(float, scale)),
                                     float(out_scale))
        check("fcdemSdfSetNormalization")

    def normalization(self):
        s, c, o = _F3(), _F3(), f32()
        lib.fcdemSdfGetNormalization(self._h, s, c, C.byref(o))
        return np.array(s, np.float32), np.array(c, np.float32), float(o.value)

    def normalize_to(self, dmap: DistanceMap) -> None:
        """Inputs scaled to [-1, 1] over the map box (one scale for all axes),
        outputs in units of the box's largest half-extent."""
        centre = 0.5 * (dmap.vmin + dmap.vmax)
        half = float(np.max(0.5 * (dmap.vmax - dmap.vmin)))
        self.set_normalization(centre, [1.0 / half] * 3, half)

    def gradient(self, samples: torch.Tensor, shapes: torch.Tensor | None = None,
                 band: float = 0.0):
        g = np.zeros(self.num_params, np.float32)
        loss = lib.fcdemSdfGradient(self._h, _p(samples), _opt(shapes), samples.shape[0],
                                    band, g.ctypes.data)
        check("fcdemSdfGradient")
        return float(loss), g

    def train(self, samples: torch.Tensor, shapes: torch.Tensor | None = None,
              epochs: int = 10, batch: int = 8192, lr: float = 2e-3, band: float = 0.0) -> float:
        loss = lib.fcdemSdfTrainSamples(self._h, _p(samples), _opt(shapes), samples.shape[0],
                                        epochs, batch, lr, band)
        check("fcdemSdfTrainSamples")
        return float(loss)

    def eval_f32(self, pts: torch.Tensor, shapes: torch.Tensor | None = None) -> torch.Tensor:
        d = torch.empty(pts.shape[0], dtype=torch.float32, device=pts.device)
        lib.fcdemSdfEvalF32(self._h, _p(pts), _opt(shapes), pts.shape[0], _p(d))
        check("fcdemSdfEvalF32")
        return d

    def infer(self, pts: torch.Tensor, shapes: torch.Tensor | None = None) -> torch.Tensor:
        d = torch.empty(pts.shape[0], dtype=torch.float32, device=pts.device)
        lib.fcdemSdfInfer(self._h, _p(pts), _opt(shapes), pts.shape[0], _p(d))
        check("fcdemSdfInfer")
        return d

    def set_tile_culling(self, lipschitz: float) -> None:
        """0: cull the map query per particle; > 0: per tile of 32 slots with
        this Lipschitz bound of the prediction (fcdemSdfSetTileCulling)."""
        lib.fcdemSdfSetTileCulling(self._h, float(lipschitz))
        check("fcdemSdfSetTileCulling")

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib.fcdemSdfDestroy(h)
            self._h = None


def samples(dmap: DistanceMap, n: int, near_fraction: float = 0.5, band: float = 0.05,
            seed: int = 7, shape: int | None = None, device="cuda"):
    """n training samples (x, y, z, distance) of the map; with `shape`, also
    the int32 shape codes."""
    s = torch.empty((n, 4), dtype=torch.float32, device=device)
    sh = torch.empty(n, dtype=torch.int32, device=device) if shape is not None else None
    lib.fcdemSdfSamples(dmap.handle, -1 if shape is None else shape, n, near_fraction, band,
                        seed, _p(s), _opt(sh))
    check("fcdemSdfSamples")
    return (s, sh) if shape is not None else s


def um_integrate_system_sdf(pos, vel, dt: float, n: int, dmap: DistanceMap, net: SdfNet,
                            skin: float, exact_counter: torch.Tensor | None = None) -> None:
    lib.fcdemUM_integrateSystemSdf(_p(pos), _p(vel), dt, n, dmap.handle, net.handle, skin,
                                   _opt(exact_counter))


def obstacle_maps(obstacles: list, cells_per_axis: int = 128, margin: float = 0.05) -> list:
    """DistanceMap of each obstacle of scenes.obstacle_set."""
    from .dem import DistanceMap
    out = []
    for ob in obstacles:
        if ob["kind"] == "torus":
            out.append(DistanceMap.torus(ob["R"], ob["r"], cells_per_axis, margin))
        else:
            out.append(DistanceMap.rounded_box(ob["h"], ob["rounding"], cells_per_axis, margin))
    return out


def shape_net(maps: list, samples_per_map: int = 500_000, hidden: int = 128, layers: int = 2,
              epochs: int = 40, batch: int = 2048, lr: float = 5e-3, band: float = 0.02,
              seed: int = 9):
    """A shape-conditioned network (3 + len(maps) inputs) trained on samples
    of every map, each with its shape code; inputs and outputs normalised by
    the largest half-extent over the maps.  Returns (net, final loss)."""
    lo = np.min([m.vmin for m in maps], axis=0)
    hi = np.max([m.vmax for m in maps], axis=0)
    half = float(np.max(np.maximum(np.abs(lo), np.abs(hi))))
    net = SdfNet(3 + len(maps), hidden, layers, seed=seed)
    net.set_normalization([0.0, 0.0, 0.0], [1.0 / half] * 3, half)
    parts, shapes = [], []
    for k, m in enumerate(maps):
        s_k, sh_k = samples(m, samples_per_map, 0.6, 0.05, seed=seed * 131 + k, shape=k)
        parts.append(s_k)
        shapes.append(sh_k)
    s = torch.cat(parts)
    sh = torch.cat(shapes)
    g = torch.Generator(device=s.device).manual_seed(seed)
    perm = torch.randperm(s.shape[0], device=s.device, generator=g)
    s, sh = s[perm].contiguous(), sh[perm].contiguous()
    loss = net.train(s, sh, epochs=epochs, batch=batch, lr=lr, band=band)
    return net, loss


def calibrate_skin(net: SdfNet, maps: list, radius: float, samples_per_map: int = 500_000,
                   seed: int = 300, shaped: bool = True, margin: float = 0.5) -> tuple:
    """The culling threshold, judged by the exact maps: on held-out samples
    of every map, p_max = the largest prediction at a point the map puts
    within one radius of the surface (or inside the obstacle), the value that
    must not be culled.  The skin is max(2 radius, p_max + margin (p_max -
    radius)); the margin covers points the samples missed.  Returns
    (skin, p_max)."""
    p_max = -1e30
    for k, m in enumerate(maps):
        if shaped:
            val, sh = samples(m, samples_per_map, 0.5, 0.03, seed=seed + k, shape=k)
        else:
            val, sh = samples(m, samples_per_map, 0.5, 0.03, seed=seed + k), None
        pred = net.infer(val, sh)
        touching = val[:, 3] < radius
        if bool(touching.any()):
            p_max = max(p_max, float(pred[touching].max()))
    return max(2.0 * radius, p_max + margin * max(p_max - radius, 0.0)), p_max


def calibrate_lipschitz(net: SdfNet, maps: list, pairs_per_map: int = 500_000,
                        seed: int = 400, shaped: bool = True, safety: float = 1.5,
                        min_step: float = 0.004, max_step: float = 0.08) -> tuple:
    """A Lipschitz bound of the network's BF16 prediction (the one the culling
    uses), measured on held-out pairs of points of every map box: x from the
    map's own samples (half of them near the surface), y = x + a step of
    random direction and length U[min_step, max_step], kept in the box.
    L = max |pred(x) - pred(y)| / |x - y|; returns (safety * L, L)."""
    g = torch.Generator(device="cuda").manual_seed(seed)
    lip = 0.0
    for k, m in enumerate(maps):
        if shaped:
            x, sh = samples(m, pairs_per_map, 0.5, 0.03, seed=seed + k, shape=k)
        else:
            x, sh = samples(m, pairs_per_map, 0.5, 0.03, seed=seed + k), None
        u = torch.randn(pairs_per_map, 3, generator=g, device="cuda")
        u = u / u.norm(dim=1, keepdim=True)
        step = min_step + (max_step - min_step) * torch.rand(pairs_per_map, 1, generator=g,
                                                             device="cuda")
        y = x.clone()
        y[:, :3] = x[:, :3] + u * step
        lo = torch.as_tensor(m.vmin, device="cuda")
        hi = torch.as_tensor(m.vmax, device="cuda")
        keep = ((y[:, :3] >= lo) & (y[:, :3] <= hi)).all(dim=1)
        x, y = x[keep].contiguous(), y[keep].contiguous()
        shk = sh[keep].contiguous() if sh is not None else None
        px, py = net.infer(x, shk), net.infer(y, shk)
        ratio = (px - py).abs() / (x[:, :3] - y[:, :3]).norm(dim=1)
        lip = max(lip, float(ratio.max()))
    return safety * lip, lip
