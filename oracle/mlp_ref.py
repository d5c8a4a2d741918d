"""CPU reference of the warm-start MLP (test infrastructure: the checker of
the device kernels, never the product path).

A dense network with tanh hidden layers and a linear output layer,
layers [(W, b), ...] with W [d_in][d_out]; the loss is the mean squared
error over the selected rows and all outputs; AdamW as the host training
used it (torch.optim.AdamW defaults: beta 0.9 / 0.999, eps 1e-8, decoupled
weight decay, bias-corrected moments).  Plain numpy, FP64, written out step
by step so that every intermediate can be compared."""
from __future__ import annotations

import numpy as np


def forward(layers, x):
    """Activations [x, h_1, ..., y]."""
    acts = [np.asarray(x, np.float64)]
    for i, (w, b) in enumerate(layers):
        z = acts[-1] @ w + b
        acts.append(np.tanh(z) if i < len(layers) - 1 else z)
    return acts


def loss_grad(layers, x, y, rows=None):
    """(loss, [(dW, db), ...]) of the mean squared error over the rows with
    rows[r] == 1 (all rows when rows is None)."""
    acts = forward(layers, x)
    sel = np.ones(len(x), bool) if rows is None else np.asarray(rows) == 1
    d = acts[-1] - y
    nout = d.shape[1]
    scale = 1.0 / (sel.sum() * nout)
    loss = float((d[sel] ** 2).sum() * scale)
    g = np.where(sel[:, None], 2.0 * scale * d, 0.0)
    grads = [None] * len(layers)
    for i in range(len(layers) - 1, -1, -1):
        if i < len(layers) - 1:
            g = g * (1.0 - acts[i + 1] ** 2)
        grads[i] = (acts[i].T @ g, g.sum(0))
        if i > 0:
            g = g @ layers[i][0].T
    return loss, grads


class AdamW:
    """torch.optim.AdamW's update for FP64 parameters."""

    def __init__(self, layers, lr, weight_decay, betas=(0.9, 0.999), eps=1e-8):
        self.lr, self.wd, self.b1, self.b2, self.eps = lr, weight_decay, betas[0], betas[1], eps
        self.m = [[np.zeros_like(w), np.zeros_like(b)] for w, b in layers]
        self.v = [[np.zeros_like(w), np.zeros_like(b)] for w, b in layers]
        self.t = 0

    def step(self, layers, grads):
        self.t += 1
        bc1 = 1.0 - self.b1 ** self.t
        bc2 = 1.0 - self.b2 ** self.t
        out = []
        for i, (pair, gpair) in enumerate(zip(layers, grads)):
            new = []
            for j in range(2):
                p, g = pair[j], gpair[j]
                m = self.m[i][j] + (1.0 - self.b1) * (g - self.m[i][j])
                v = self.v[i][j] * self.b2 + (1.0 - self.b2) * g * g
                self.m[i][j], self.v[i][j] = m, v
                p = p * (1.0 - self.lr * self.wd)
                new.append(p + (-self.lr / bc1) * (m / (np.sqrt(v) / np.sqrt(bc2) + self.eps)))
            out.append((new[0], new[1]))
        return out


def train(layers, x, y, rows, epochs, lr, weight_decay, eval_every=20):
    """Full-batch training as the device entry point runs it: per epoch the
    training loss (before the step), the AdamW step, and every eval_every
    epochs (and after the last) the held-out loss, keeping the parameters of
    the lowest one.  Returns (final, best, losses, (best held-out, its
    training loss))."""
    opt = AdamW(layers, lr, weight_decay)
    rows = np.asarray(rows)
    held = (rows == 0).astype(np.uint8) if rows is not None else None
    best, bestp, losses = (np.inf, np.inf), layers, []
    for ep in range(epochs):
        loss, grads = loss_grad(layers, x, y, rows)
        losses.append(loss)
        layers = opt.step(layers, grads)
        if held is not None and held.any() and (ep % eval_every == 0 or ep == epochs - 1):
            vl, _ = loss_grad(layers, x, y, held)
            if vl < best[0]:
                best, bestp = (vl, loss), layers
    return layers, bestp, np.array(losses), best


def bf16_round(a):
    """Round to the nearest BF16 value (ties to even) of the FP32 value of
    each entry, returned as float64: the weights the BF16 network multiplies
    with.  Bit form: the FP32 pattern plus 0x7FFF plus the lowest kept bit,
    cut to the upper 16 bits (finite inputs)."""
    f = np.ascontiguousarray(a, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def layers16(layers):
    """The BF16-weight network of FP32 master layers: weights rounded, biases
    kept in FP32."""
    return [(bf16_round(w), np.asarray(np.float32(b), np.float64)) for w, b in layers]


def forward16(layers, x):
    """Activations of the BF16-weight network (FP64 arithmetic on the rounded
    weights; the device runs the same products in FP32)."""
    return forward(layers16(layers), np.asarray(np.float32(x), np.float64))


def loss_grad16(layers, x, y, rows=None):
    """Loss and gradient of the BF16-weight network with respect to its
    weights, which the device applies to the FP32 masters."""
    return loss_grad(layers16(layers), np.asarray(np.float32(x), np.float64),
                     np.asarray(np.float32(y), np.float64), rows)
