"""CPU oracle of the cooling surrogate's network (test infrastructure only).

The surrogate has no counterpart in the reference: it is this build's
replacement of the per-cell cooling integration (source/cooling.f90:64-112).
Its network is a 3-64-64-64-1 multilayer perceptron with SiLU activations,
packed as W1[64][3] b1[64] W2[64][64] b2[64] W3[64][64] b3[64] W4[64] b4
(8641 FP32 parameters).  This module restates the forward pass and the
backward pass of the mean-squared-error loss in numpy FP64, optionally with
the GPU kernels' roundings to BF16:

* the weights of the hidden layers 2 and 3 and every SiLU activation that
  feeds a tensor-core product are rounded to BF16 (round to nearest even);
  the 3 -> 64 input and 64 -> 1 output layers are unrounded (FP32 on the
  GPU);
* in the backward pass the layer-3/2 deltas are rounded to BF16 where they
  feed the tensor-core products dW = dZ^T H and dH = dZ W; the layer-4 and
  layer-1 weight gradients and all bias gradients use the unrounded deltas.

With ``bf16=False`` the functions are the plain FP64 network, whose gradient
is pinned against central finite differences in the CPU tests; with
``bf16=True`` they are the reference the GPU gradient and inference are
checked against.
"""
from __future__ import annotations

import numpy as np

IN, HID = 3, 64
OFF_W1 = 0
OFF_B1 = OFF_W1 + HID * IN
OFF_W2 = OFF_B1 + HID
OFF_B2 = OFF_W2 + HID * HID
OFF_W3 = OFF_B2 + HID
OFF_B3 = OFF_W3 + HID * HID
OFF_W4 = OFF_B3 + HID
OFF_B4 = OFF_W4 + HID
NPARAM = OFF_B4 + 1


def bf16(x) -> np.ndarray:
    """Round to BF16 (nearest even) through FP32, returned as float64."""
    f = np.ascontiguousarray(x, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(P):
    P = np.asarray(P, dtype=np.float64)
    W1 = P[OFF_W1:OFF_B1].reshape(HID, IN)
    b1 = P[OFF_B1:OFF_W2]
    W2 = P[OFF_W2:OFF_B2].reshape(HID, HID)
    b2 = P[OFF_B2:OFF_W3]
    W3 = P[OFF_W3:OFF_B3].reshape(HID, HID)
    b3 = P[OFF_B3:OFF_W4]
    W4 = P[OFF_W4:OFF_B4]
    b4 = P[OFF_B4]
    return W1, b1, W2, b2, W3, b3, W4, b4


def _sig(z):
    return 1.0 / (1.0 + np.exp(-z))


def silu(z):
    return z * _sig(z)


def dsilu(z):
    s = _sig(z)
    return s * (1.0 + z * (1.0 - s))


def forward(P, X, bf16_round: bool = True):
    """y for normalised features X [n,3]; also returns the pre-activations."""
    r = bf16 if bf16_round else (lambda a: np.asarray(a, dtype=np.float64))
    W1, b1, W2, b2, W3, b3, W4, b4 = unpack(P)
    x = np.asarray(X, dtype=np.float64)
    z1 = x @ W1.T + b1
    z2 = r(silu(z1)) @ r(W2).T + b2
    z3 = r(silu(z2)) @ r(W3).T + b3
    y = silu(z3) @ W4 + b4
    return y, (x, z1, z2, z3)


def loss_grad(P, X, Y, bf16_round: bool = True, wt=None):
    """(loss sum |w| e^2 / n, gradient [8641]) with the GPU kernel's roundings;
    e = y - t, or min(y - t, 0) where w < 0 (one-sided target); w = 1 when wt
    is None."""
    r = bf16 if bf16_round else (lambda a: np.asarray(a, dtype=np.float64))
    W1, b1, W2, b2, W3, b3, W4, b4 = unpack(P)
    Y = np.asarray(Y, dtype=np.float64)
    n = Y.size
    y, (x, z1, z2, z3) = forward(P, X, bf16_round)
    w = np.ones(n) if wt is None else np.asarray(wt, dtype=np.float64)
    e = y - Y
    e = np.where(w < 0, np.minimum(e, 0.0), e)
    w = np.abs(w)
    loss = float(np.sum(w * e * e) / n)
    dy = 2.0 * w * e / n
    g = np.zeros(NPARAM)
    g[OFF_B4] = dy.sum()
    g[OFF_W4:OFF_B4] = dy @ silu(z3)
    d3 = dy[:, None] * W4[None, :] * dsilu(z3)
    g[OFF_B3:OFF_W4] = d3.sum(0)
    g[OFF_W3:OFF_B3] = (r(d3).T @ r(silu(z2))).ravel()
    d2 = (r(d3) @ r(W3)) * dsilu(z2)
    g[OFF_B2:OFF_W3] = d2.sum(0)
    g[OFF_W2:OFF_B2] = (r(d2).T @ r(silu(z1))).ravel()
    d1 = (r(d2) @ r(W2)) * dsilu(z1)
    g[OFF_B1:OFF_W2] = d1.sum(0)
    g[OFF_W1:OFF_B1] = (d1.T @ x).ravel()
    return loss, g


def init_params(seed: int = 0) -> np.ndarray:
    """Glorot-uniform weights, zero biases, b4 = 1 (FP32)."""
    rng = np.random.default_rng(seed)
    P = np.zeros(NPARAM, dtype=np.float32)

    def fill(off, fo, fi):
        a = np.sqrt(6.0 / (fi + fo))
        P[off:off + fo * fi] = rng.uniform(-a, a, fo * fi)

    fill(OFF_W1, HID, IN)
    fill(OFF_W2, HID, HID)
    fill(OFF_W3, HID, HID)
    fill(OFF_W4, 1, HID)
    P[OFF_B4] = 1.0
    return P
