"""CPU restatement of the learned cost model's network -- TEST INFRASTRUCTURE ONLY.

The network ``tensororder_gb300/csrc/togb_mlp.cu`` runs on the GPU: an MLP
F -> H -> H -> 1 with ReLU hidden layers, mean squared error, parameters in
one vector ``W1[F][H] b1[H] W2[H][H] b2[H] W3[H] b3``.  This module computes
the same forward pass, loss and gradients in float64 numpy, so the tests can
check the device gradients against it (the reference has no learned model;
its cost model is the FLOP/memory estimate of
``contraction_methods/contraction_tree.pyx:382-496``).
"""
from __future__ import annotations

import numpy as np


def unpack(p, F, H):
    p = np.asarray(p, dtype=np.float64)
    i = 0

    def take(n, shape):
        nonlocal i
        out = p[i:i + n].reshape(shape)
        i += n
        return out

    W1 = take(F * H, (F, H))
    b1 = take(H, (H,))
    W2 = take(H * H, (H, H))
    b2 = take(H, (H,))
    W3 = take(H, (H,))
    b3 = take(1, ())
    assert i == p.size
    return W1, b1, W2, b2, W3, b3


def forward(p, F, H, x):
    W1, b1, W2, b2, W3, b3 = unpack(p, F, H)
    x = np.asarray(x, dtype=np.float64)
    z1 = x @ W1 + b1
    a1 = np.maximum(z1, 0)
    z2 = a1 @ W2 + b2
    a2 = np.maximum(z2, 0)
    return a2 @ W3 + b3, (x, a1, a2)


def loss_grad(p, F, H, x, target):
    W1, b1, W2, b2, W3, b3 = unpack(p, F, H)
    y, (x, a1, a2) = forward(p, F, H, x)
    B = x.shape[0]
    d = y - np.asarray(target, dtype=np.float64)
    loss = float(np.mean(d * d))
    dy = 2.0 * d / B
    gW3 = a2.T @ dy
    gb3 = dy.sum()
    dz2 = np.outer(dy, W3) * (a2 > 0)
    gW2 = a1.T @ dz2
    gb2 = dz2.sum(0)
    dz1 = (dz2 @ W2.T) * (a1 > 0)
    gW1 = x.T @ dz1
    gb1 = dz1.sum(0)
    g = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3, [gb3]])
    return loss, g
