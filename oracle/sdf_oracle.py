"""FP64 CPU oracle of the neural-SDF network's forward pass, loss and gradient.

Test infrastructure only: the tests import it to check the GPU training
kernels' gradients and predictions; nothing on the product path does.

Network (the library's fcdemSdf* calls): input u = ((x, y, z) - shift) * scale
followed by a one-hot shape code (inputs - 3 entries), `layers` hidden layers
h_l = silu(W_l h_{l-1} + b_l) of width H, output y = wOut . h_L + bOut, and
the distance d = y * outScale.  Loss over n samples (x, y, z, d):
    L = sum_s w_s (y_s - d_s / outScale)^2 / n,  w_s = 10 if |d_s| < band else 1.
Parameter vector: W0 [H][D], b0, per further hidden layer W [H][H], b, then
wOut [H], bOut (row-major [out][in]).
"""
from __future__ import annotations

import numpy as np


def layout(inputs: int, hidden: int, layers: int) -> dict:
    off = 0
    lay = {"D": inputs, "H": hidden, "L": layers, "W": [], "b": []}
    shapes = [(hidden, inputs)] + [(hidden, hidden)] * (layers - 1)
    for shp in shapes:
        lay["W"].append((off, shp))
        off += shp[0] * shp[1]
        lay["b"].append(off)
        off += hidden
    lay["wo"] = off
    off += hidden
    lay["bo"] = off
    off += 1
    lay["total"] = off
    return lay


def unpack(p: np.ndarray, lay: dict):
    p = np.asarray(p, np.float64)
    H = lay["H"]
    Ws = [p[o:o + r * c].reshape(r, c) for o, (r, c) in lay["W"]]
    bs = [p[o:o + H] for o in lay["b"]]
    return Ws, bs, p[lay["wo"]:lay["wo"] + H], p[lay["bo"]]


def _sig(z):
    return 1.0 / (1.0 + np.exp(-z))


def inputs_of(pts: np.ndarray, shapes, lay: dict, shift, scale) -> np.ndarray:
    pts = np.asarray(pts, np.float64)
    n = pts.shape[0]
    X = np.zeros((n, lay["D"]))
    X[:, :3] = (pts[:, :3] - np.asarray(shift, np.float64)) * np.asarray(scale, np.float64)
    if shapes is not None and lay["D"] > 3:
        sh = np.asarray(shapes)
        ok = (sh >= 0) & (sh < lay["D"] - 3)
        X[np.nonzero(ok)[0], 3 + sh[ok]] = 1.0
    return X


def forward(p, lay, pts, shapes=None, shift=(0, 0, 0), scale=(1, 1, 1), out_scale=1.0):
    """Distance predictions (FP64)."""
    Ws, bs, wo, bo = unpack(p, lay)
    h = inputs_of(pts, shapes, lay, shift, scale)
    for W, b in zip(Ws, bs):
        z = h @ W.T + b
        h = z * _sig(z)
    return (h @ wo + bo) * out_scale


def loss_and_grad(p, lay, samples, shapes=None, band=0.0, shift=(0, 0, 0), scale=(1, 1, 1),
                  out_scale=1.0):
    """(loss, gradient) in FP64 for samples (n, 4) = (x, y, z, d)."""
    samples = np.asarray(samples, np.float64)
    n = samples.shape[0]
    Ws, bs, wo, bo = unpack(p, lay)
    X = inputs_of(samples, shapes, lay, shift, scale)
    zs, hs = [], [X]
    h = X
    for W, b in zip(Ws, bs):
        z = h @ W.T + b
        zs.append(z)
        h = z * _sig(z)
        hs.append(h)
    y = h @ wo + bo
    d = samples[:, 3]
    t = d / out_scale
    w = np.where(np.abs(d) < band, 10.0, 1.0)
    r = y - t
    loss = float(np.sum(w * r * r) / n)
    dy = 2.0 * w * r / n
    g = np.zeros(lay["total"])
    g[lay["wo"]:lay["wo"] + lay["H"]] = hs[-1].T @ dy
    g[lay["bo"]] = dy.sum()
    delta = np.outer(dy, wo)
    for l in range(len(Ws) - 1, -1, -1):
        s = _sig(zs[l])
        delta = delta * (s * (1.0 + zs[l] * (1.0 - s)))
        o, (rr, cc) = lay["W"][l]
        g[o:o + rr * cc] = (delta.T @ hs[l]).reshape(-1)
        g[lay["b"][l]:lay["b"][l] + lay["H"]] = delta.sum(axis=0)
        delta = delta @ Ws[l]
    return loss, g
