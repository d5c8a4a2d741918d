"""The CPU reference of the warm-start MLP (oracle/mlp_ref.py) against torch
on the CPU: forward, the gradient of the masked mean squared error (autograd)
and a run of AdamW steps (torch.optim.AdamW), FP64.  It is the checker the
device kernels are held to."""
import numpy as np
import pytest

import mlp_ref as M

torch = pytest.importorskip("torch")


def _net(rng, dims):
    return [(rng.normal(size=(a, b)) / np.sqrt(a), rng.normal(size=b) * 0.1) for a, b in zip(dims[:-1], dims[1:])]


def _torch(layers):
    ps = []
    for w, b in layers:
        ps += [torch.tensor(w, requires_grad=True), torch.tensor(b, requires_grad=True)]
    return ps


def _tfwd(ps, x):
    h = x
    n = len(ps) // 2
    for i in range(n):
        h = h @ ps[2 * i] + ps[2 * i + 1]
        if i < n - 1:
            h = torch.tanh(h)
    return h


def test_forward_and_gradient_match_autograd():
    rng = np.random.default_rng(1)
    dims = [11, 16, 16, 6]
    layers = _net(rng, dims)
    x, y = rng.normal(size=(37, 11)), rng.normal(size=(37, 6))
    rows = (rng.random(37) < 0.7).astype(np.uint8)
    loss, grads = M.loss_grad(layers, x, y, rows)
    ps = _torch(layers)
    sel = torch.tensor(rows == 1)
    tl = ((_tfwd(ps, torch.tensor(x))[sel] - torch.tensor(y)[sel]) ** 2).mean()
    tl.backward()
    assert abs(loss - tl.item()) < 1e-14 * abs(tl.item())
    for i, (gw, gb) in enumerate(grads):
        assert np.abs(gw - ps[2 * i].grad.numpy()).max() < 1e-14 * np.abs(gw).max()
        assert np.abs(gb - ps[2 * i + 1].grad.numpy()).max() < 1e-14 * np.abs(gb).max()
    assert np.allclose(M.forward(layers, x)[-1], _tfwd(ps, torch.tensor(x)).detach().numpy(), rtol=0, atol=1e-14)


def test_adamw_matches_torch():
    rng = np.random.default_rng(2)
    dims = [7, 12, 12, 4]
    layers = _net(rng, dims)
    x, y = rng.normal(size=(25, 7)), rng.normal(size=(25, 4))
    opt = M.AdamW(layers, 2e-3, 1e-4)
    ps = _torch(layers)
    topt = torch.optim.AdamW(ps, lr=2e-3, weight_decay=1e-4)
    for _ in range(25):
        _, grads = M.loss_grad(layers, x, y)
        layers = opt.step(layers, grads)
        topt.zero_grad()
        ((_tfwd(ps, torch.tensor(x)) - torch.tensor(y)) ** 2).mean().backward()
        topt.step()
    for i, (w, b) in enumerate(layers):
        assert np.abs(w - ps[2 * i].detach().numpy()).max() < 1e-13
        assert np.abs(b - ps[2 * i + 1].detach().numpy()).max() < 1e-13


def test_train_keeps_the_best_held_out_epoch():
    rng = np.random.default_rng(3)
    layers = _net(rng, [5, 8, 3])
    x, y = rng.normal(size=(40, 5)), rng.normal(size=(40, 3))
    rows = np.array([1] * 30 + [0] * 10, np.uint8)
    final, best, losses, (bv, bt) = M.train(layers, x, y, rows, 60, 1e-2, 0.0, eval_every=20)
    assert len(losses) == 60 and losses[-1] < losses[0]
    held = (rows == 0).astype(np.uint8)
    vals = {}
    opt = M.AdamW(layers, 1e-2, 0.0)
    cur = layers
    for ep in range(60):
        _, g = M.loss_grad(cur, x, y, rows)
        cur = opt.step(cur, g)
        if ep % 20 == 0 or ep == 59:
            vals[ep] = M.loss_grad(cur, x, y, held)[0]
    assert abs(bv - min(vals.values())) < 1e-15
    assert np.array_equal(final[0][0], cur[0][0])


def test_device_element_logic_on_the_host(tmp_path):
    # mlp_dev.cuh (the bodies of the device kernels) compiled for the host and
    # driven like skkr_gpu_mlp_grad: the loss and packed gradient equal the
    # reference's, and one AdamW step equals the reference's step
    import ctypes
    import os
    import subprocess
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    so = str(tmp_path / "libmlp.so")
    subprocess.run(["g++", "-O2", "-shared", "-fPIC", "-o", so, os.path.join(root, "tests", "harness", "mlp_host.cpp")],
                   check=True)
    L = ctypes.CDLL(so)
    P, I, D = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
    L.mlp_grad_eval.argtypes = [I, P, P, I, P, P, P, P, P]
    L.mlp_adamw_eval.argtypes = [ctypes.c_longlong, P, P, P, P, D, D, D, D]
    rng = np.random.default_rng(8)
    dims = [19, 32, 32, 14]
    layers = _net(rng, dims)
    x, y = rng.normal(size=(90, 19)), rng.normal(size=(90, 14))
    rows = (rng.random(90) < 0.8).astype(np.uint8)
    d = np.array(dims, np.int32)
    params = np.concatenate([np.concatenate([w.ravel(), b]) for w, b in layers])
    grad = np.zeros_like(params)
    loss = np.zeros(1)
    L.mlp_grad_eval(3, d.ctypes.data, params.ctypes.data, 90, x.ctypes.data, y.ctypes.data, rows.ctypes.data,
                    loss.ctypes.data, grad.ctypes.data)
    lr_, gr = M.loss_grad(layers, x, y, rows)
    ref = np.concatenate([np.concatenate([gw.ravel(), gb]) for gw, gb in gr])
    assert abs(loss[0] - lr_) < 1e-14 * lr_
    assert np.abs(grad - ref).max() < 1e-13 * np.abs(ref).max()
    m, v, p = np.zeros_like(params), np.zeros_like(params), params.copy()
    bc1, bc2 = 1 - 0.9, 1 - 0.999
    L.mlp_adamw_eval(len(p), p.ctypes.data, grad.ctypes.data, m.ctypes.data, v.ctypes.data, 2e-3, 1e-4, 2e-3 / bc1,
                     np.sqrt(bc2))
    step = M.AdamW(layers, 2e-3, 1e-4).step(layers, gr)
    refp = np.concatenate([np.concatenate([w.ravel(), b]) for w, b in step])
    assert np.abs(p - refp).max() < 1e-13 * np.abs(refp).max()
