"""The warm-start MLP on the device (skkr_gpu_mlp_*: this library's forward,
backward and AdamW kernels, FP64) against the CPU reference oracle/mlp_ref.py
(itself checked against torch autograd and torch.optim.AdamW): outputs,
gradients of the masked loss and a training run with the held-out best
epoch."""
import numpy as np
import pytest

import mlp_ref as M
from skkr_budapest_gb300 import native

pytestmark = pytest.mark.gpu


def _net(rng, dims):
    return [(rng.normal(size=(a, b)) / np.sqrt(a), rng.normal(size=b) * 0.1) for a, b in zip(dims[:-1], dims[1:])]


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


DIMS = [19, 64, 64, 14]


def test_forward_matches_reference():
    rng = np.random.default_rng(4)
    layers = _net(rng, DIMS)
    x = rng.normal(size=(300, DIMS[0]))
    assert _rel(native.mlp_forward(layers, x), M.forward(layers, x)[-1]) < 1e-13


def test_gradient_matches_reference():
    rng = np.random.default_rng(5)
    layers = _net(rng, DIMS)
    x, y = rng.normal(size=(257, DIMS[0])), rng.normal(size=(257, DIMS[-1]))
    rows = (rng.random(257) < 0.8).astype(np.uint8)
    lg, gg = native.mlp_grad(layers, x, y, rows)
    lr_, gr = M.loss_grad(layers, x, y, rows)
    assert abs(lg - lr_) < 1e-13 * lr_
    for (gw, gb), (rw, rb) in zip(gg, gr):
        assert _rel(gw, rw) < 1e-12 and _rel(gb, rb) < 1e-12


def test_training_matches_reference():
    rng = np.random.default_rng(6)
    layers = _net(rng, DIMS)
    x = rng.normal(size=(400, DIMS[0]))
    y = np.tanh(x[:, :DIMS[-1]]) + 0.05 * rng.normal(size=(400, DIMS[-1]))
    rows = np.array([1] * 340 + [0] * 60, np.uint8)
    fg, bg, lg, (vg, tg) = native.mlp_train(layers, x, y, rows, 60, 2e-3, 1e-4, eval_every=20)
    fr, br, lr_, (vr, tr) = M.train(layers, x, y, rows, 60, 2e-3, 1e-4, eval_every=20)
    assert _rel(lg, lr_) < 1e-10 and lg[-1] < lg[0]
    assert abs(vg - vr) < 1e-10 * vr and abs(tg - tr) < 1e-10 * tr
    for (a, b), (c, d) in zip(fg + bg, fr + br):
        assert _rel(a, c) < 1e-9 and _rel(b, d) < 1e-9
