"""CPU restatement of the learned KT corrector -- TEST INFRASTRUCTURE ONLY.

The network corrects one coarse KT step of a t-column towards the result of
the fully sub-cycled KT step.  Only ``tests/`` may import this module, as the
checker of the CUDA forward/backward kernels; the product never does.

Network (per column, t along the last axis, 'same' zero padding of 2 per
layer, so no layer mixes samples of different columns):
    h1 = GELU(conv(x,  W1[64,1,5])  + b1)
    h2 = GELU(conv(h1, W2[64,64,5]) + b2)
    h3 = GELU(conv(h2, W3[64,64,5]) + b3)
    y  =      conv(h3, W4[1,64,5])  + b4
    conv(x, W)[o, t] = sum_i sum_j W[o, i, j] x[i, t + j - 2]
GELU(z) = z/2 (1 + tanh(sqrt(2/pi) (z + 0.044715 z^3))) (the tanh form).
Loss: masked mean squared error.

There is no reference implementation of this part (the reference solver has
no learned component); the KT targets come from the reference's KT scheme
(``_kt_flux``/``_kt_flux_adaptive``, angular_spectrum_solver.py:833-859), which
the main oracle restates.  This module is pinned by finite differences
(``tests/test_corrector_oracle.py``), not by golden vectors.
"""
from __future__ import annotations

import math

import numpy as np

K = 5
PAD = 2
CH = 64


def bf16(a):
    """Round to bfloat16 (nearest, ties to even) and back to float32."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    out = r.astype(np.uint32).view(np.float32)
    return np.where(np.isnan(a), a, out)


_C = math.sqrt(2.0 / math.pi)


def gelu(z):
    """GELU in its tanh form."""
    return 0.5 * z * (1.0 + np.tanh(_C * (z + 0.044715 * z ** 3)))


def gelu_grad(z):
    t = np.tanh(_C * (z + 0.044715 * z ** 3))
    return 0.5 * (1.0 + t) + 0.5 * z * (1.0 - t * t) * _C * (1.0 + 3 * 0.044715 * z * z)


def conv(x, W, b=None):
    """x (B, Ci, T), W (Co, Ci, K) -> (B, Co, T), zero padding PAD."""
    B, Ci, T = x.shape
    xp = np.zeros((B, Ci, T + 2 * PAD), dtype=np.float64)
    xp[:, :, PAD:PAD + T] = x
    out = np.zeros((B, W.shape[0], T), dtype=np.float64)
    for j in range(K):
        out += np.einsum("oi,bit->bot", W[:, :, j].astype(np.float64), xp[:, :, j:j + T])
    if b is not None:
        out += b.astype(np.float64)[None, :, None]
    return out


def conv_grad_input(dy, W, T):
    """d conv / d x: (B, Co, T) -> (B, Ci, T)."""
    B = dy.shape[0]
    dxp = np.zeros((B, W.shape[1], T + 2 * PAD), dtype=np.float64)
    for j in range(K):
        dxp[:, :, j:j + T] += np.einsum("oi,bot->bit", W[:, :, j].astype(np.float64), dy)
    return dxp[:, :, PAD:PAD + T]


def conv_grad_weight(dy, x):
    """d conv / d W: (Co, Ci, K)."""
    B, Ci, T = x.shape
    xp = np.zeros((B, Ci, T + 2 * PAD), dtype=np.float64)
    xp[:, :, PAD:PAD + T] = x
    dW = np.zeros((dy.shape[1], Ci, K), dtype=np.float64)
    for j in range(K):
        dW[:, :, j] = np.einsum("bot,bit->oi", dy, xp[:, :, j:j + T])
    return dW


NAMES = ["W1", "b1", "W2", "b2", "W3", "b3", "W4", "b4"]


def forward(x, P):
    """x (B, T) -> y (B, T) and the cache of pre-activations."""
    x = np.asarray(x, np.float64)[:, None, :]
    z1 = conv(x, P["W1"], P["b1"])
    h1 = gelu(z1)
    z2 = conv(h1, P["W2"], P["b2"])
    h2 = gelu(z2)
    z3 = conv(h2, P["W3"], P["b3"])
    h3 = gelu(z3)
    y = conv(h3, P["W4"], P["b4"])[:, 0, :]
    return y, dict(x=x, z1=z1, h1=h1, z2=z2, h2=h2, z3=z3, h3=h3)


def loss_and_grads(x, target, mask, P):
    """Masked MSE sum(mask (y - target)^2) / sum(mask) and its gradients."""
    y, c = forward(x, P)
    m = np.asarray(mask, np.float64)
    n = max(m.sum(), 1.0)
    r = (y - target) * m
    loss = float((r * r).sum() / n)
    dy = (2.0 / n * r)[:, None, :]
    T = y.shape[-1]
    g = {}
    g["W4"] = conv_grad_weight(dy, c["h3"])
    g["b4"] = dy.sum(axis=(0, 2))
    dz3 = conv_grad_input(dy, P["W4"], T) * gelu_grad(c["z3"])
    g["W3"] = conv_grad_weight(dz3, c["h2"])
    g["b3"] = dz3.sum(axis=(0, 2))
    dz2 = conv_grad_input(dz3, P["W3"], T) * gelu_grad(c["z2"])
    g["W2"] = conv_grad_weight(dz2, c["h1"])
    g["b2"] = dz2.sum(axis=(0, 2))
    dz1 = conv_grad_input(dz2, P["W2"], T) * gelu_grad(c["z1"])
    g["W1"] = conv_grad_weight(dz1, c["x"])
    g["b1"] = dz1.sum(axis=(0, 2))
    return loss, g


def loss_only(x, target, mask, P):
    y, _ = forward(x, P)
    m = np.asarray(mask, np.float64)
    r = (y - target) * m
    return float((r * r).sum() / max(m.sum(), 1.0))
