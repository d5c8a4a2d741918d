"""The BF16-weight warm-start network on the device (FP32 masters, BF16
weights in the products, FP32 activations and accumulation) against the
numpy reference of the same network (oracle/mlp_ref.py: FP64 arithmetic on
the BF16-rounded weights): outputs and gradients to the FP32 accumulation
error, and a short training run that lowers the loss like the reference."""
import numpy as np
import pytest

import mlp_ref as R
from skkr_budapest_gb300 import native as N

pytestmark = pytest.mark.gpu


def _net(dims, seed):
    rng = np.random.default_rng(seed)
    return [(np.float32(rng.uniform(-1, 1, (a, b)) / np.sqrt(a)), np.float32(rng.uniform(-0.1, 0.1, b)))
            for a, b in zip(dims[:-1], dims[1:])]


def rel(a, b):
    return np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(b)


@pytest.mark.parametrize("dims,n", [([118, 256, 256, 256, 40], 3000), ([7, 33, 5], 257)])
def test_forward_and_gradient_match_the_reference(dims, n):
    rng = np.random.default_rng(1)
    layers = _net(dims, 2)
    x = np.float32(rng.normal(size=(n, dims[0])))
    y = np.float32(rng.normal(size=(n, dims[-1])) * 0.3)
    rows = (rng.random(n) < 0.8).astype(np.uint8)
    assert rel(N.mlp16_forward(layers, x), R.forward16(layers, x)[-1]) < 2e-6
    loss, g = N.mlp16_grad(layers, x, y, rows)
    lr_, gr = R.loss_grad16(layers, x, y, rows)
    assert abs(loss - lr_) / lr_ < 1e-5
    for (dw, db), (rw, rb) in zip(g, gr):
        assert rel(dw, rw) < 1e-4 and rel(db, rb) < 1e-4


def test_bf16_weights_are_what_the_products_read():
    # a weight between two BF16 values: the forward pass must see the rounded one
    w = np.float32([[1.0 + 2.0 ** -8]])      # halfway between 1 and 1 + 2^-7: ties to even, 1.0
    b = np.float32([0.0])
    x = np.float32([[3.0]])
    assert N.mlp16_forward([(w, b)], x)[0, 0] == 3.0
    w2 = np.float32([[1.0 + 3 * 2.0 ** -9]])  # rounds up to 1 + 2^-7
    assert N.mlp16_forward([(w2, b)], x)[0, 0] == np.float32(3.0 * (1.0 + 2.0 ** -7))


def test_training_lowers_the_loss_like_the_reference():
    rng = np.random.default_rng(4)
    dims = [6, 64, 64, 64, 3]
    x = np.float32(rng.normal(size=(2048, 6)))
    y = np.float32(np.tanh(x[:, :3] * x[:, 3:]) * 0.5)
    rows = (np.arange(2048) % 10 != 0).astype(np.uint8)
    layers = _net(dims, 5)
    fin, best, tl, (vbest, _) = N.mlp16_train(layers, x, y, rows, 400, 3e-3, 1e-4, eval_every=10)
    assert tl[-1] < 0.1 * tl[0]
    assert np.isfinite(vbest) and vbest < 0.2 * tl[0]
    # the first step equals the reference's AdamW step on the same gradient
    f1, _, tl1, _ = N.mlp16_train(layers, x, y, rows, 1, 3e-3, 1e-4, eval_every=0)
    _, g = R.loss_grad16(layers, x, y, rows)
    ref = R.AdamW([(np.float64(w), np.float64(b)) for w, b in layers], 3e-3, 1e-4).step(
        [(np.float64(w), np.float64(b)) for w, b in layers], g)
    for (w, b), (rw, rb) in zip(f1, ref):
        assert np.abs(w - rw).max() < 1e-5 and np.abs(b - rb).max() < 1e-5


def test_device_resident_network_equals_the_one_call_forward():
    """skkr_gpu_mlp16_load / infer: parameters uploaded once, then row blocks
    of any size up to the handle's limit, equal to the one-call forward."""
    rng = np.random.default_rng(6)
    layers = _net([30, 64, 64, 10], 3)
    net = N.Mlp16Net(layers, maxrows=16)
    try:
        for n in (1, 4, 16):
            x = np.float32(rng.normal(size=(n, 30)))
            assert np.array_equal(net(x), N.mlp16_forward(layers, x))
        with pytest.raises(N.SkkrError):
            net(np.zeros((17, 30), np.float32))
    finally:
        net.close()
