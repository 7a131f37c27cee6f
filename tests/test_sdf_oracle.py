"""The FP64 neural-SDF oracle: its analytic gradient against central finite
differences, and its parameter layout."""
import numpy as np
import pytest

from oracle import sdf_oracle as so


@pytest.mark.parametrize("inputs,hidden,layers", [(3, 16, 3), (11, 16, 2)])
def test_oracle_gradient_matches_finite_differences(inputs, hidden, layers):
    rng = np.random.default_rng(3)
    lay = so.layout(inputs, hidden, layers)
    p = rng.normal(0.0, 0.4, lay["total"])
    n = 40
    samples = np.concatenate([rng.uniform(-1, 1, (n, 3)), rng.uniform(-0.3, 0.3, (n, 1))], 1)
    shapes = rng.integers(0, max(inputs - 3, 1), n) if inputs > 3 else None
    kw = dict(band=0.1, shift=(0.1, -0.2, 0.05), scale=(1.5, 1.5, 1.5), out_scale=0.7)
    loss, g = so.loss_and_grad(p, lay, samples, shapes, **kw)
    idx = rng.choice(lay["total"], 60, replace=False)
    h = 1e-6
    for i in idx:
        e = np.zeros_like(p)
        e[i] = h
        lp, _ = so.loss_and_grad(p + e, lay, samples, shapes, **kw)
        lm, _ = so.loss_and_grad(p - e, lay, samples, shapes, **kw)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 + 1e-5 * abs(fd), (i, fd, g[i])
    # the forward pass agrees with the loss's prediction
    y = so.forward(p, lay, samples, shapes, kw["shift"], kw["scale"], kw["out_scale"])
    r = y / kw["out_scale"] - samples[:, 3] / kw["out_scale"]
    w = np.where(np.abs(samples[:, 3]) < kw["band"], 10.0, 1.0)
    assert np.isclose(loss, np.sum(w * r * r) / n)


def test_layout_sizes():
    assert so.layout(3, 64, 3)["total"] == 64 * 3 + 64 + 2 * (64 * 64 + 64) + 64 + 1
    assert so.layout(11, 128, 2)["total"] == 128 * 11 + 128 + 128 * 128 + 128 + 128 + 1
