"""FP64 CPU reference of the surrogate MLP (forward, loss, gradients).

TEST INFRASTRUCTURE ONLY: the tests compare the GPU surrogate kernels with
it.  Architecture: nin -> hidden (x nhidden, GELU, tanh form) -> nout,
MSE loss over all outputs, parameters layer by layer as W[out][in] then
b[out] (the layout of sed_sur_get_weights).
"""
from __future__ import annotations

import numpy as np

K0 = 0.7978845608028654
K1 = 0.044715


def gelu(z):
    return 0.5 * z * (1.0 + np.tanh(K0 * (z + K1 * z ** 3)))


def gelu_grad(z):
    t = np.tanh(K0 * (z + K1 * z ** 3))
    return 0.5 * (1.0 + t) + 0.5 * z * (1.0 - t * t) * K0 * (1.0 + 3.0 * K1 * z * z)


def layer_shapes(nin, nout, hidden, nhidden):
    dims = [nin] + [hidden] * nhidden + [nout]
    return [(dims[i + 1], dims[i]) for i in range(len(dims) - 1)]


def unpack(params, shapes):
    out, o = [], 0
    for (r, c) in shapes:
        W = params[o:o + r * c].reshape(r, c)
        o += r * c
        b = params[o:o + r]
        o += r
        out.append((W, b))
    return out


def forward(params, shapes, x, bf16=False):
    """Outputs, pre-activations and layer inputs.  bf16: each hidden
    activation is rounded to BF16 where the GPU stores it (the products
    themselves stay FP64)."""
    layers = unpack(np.asarray(params, dtype=np.float64), shapes)
    a = np.asarray(x, dtype=np.float64)
    zs, acts = [], [a]
    for i, (W, b) in enumerate(layers):
        z = a @ W.T + b
        zs.append(z)
        if i < len(layers) - 1:
            a = gelu(z)
            if bf16:
                a = bf16_round(a)
            acts.append(a)
        else:
            a = z
    return a, zs, acts


def loss_and_grads(params, shapes, x, y, bf16=False):
    """MSE loss and the flat gradient.  bf16: the output gradient and each
    back-propagated gradient are rounded to BF16 where the GPU stores them,
    and the activations as in forward(bf16=True)."""
    yhat, zs, acts = forward(params, shapes, x, bf16=bf16)
    m, nout = yhat.shape
    d = yhat - y
    loss = float(np.sum(d * d) / (m * nout))
    dz = 2.0 * d / (m * nout)
    if bf16:
        dz = bf16_round(dz)
    layers = unpack(np.asarray(params, dtype=np.float64), shapes)
    grads = [None] * len(layers)
    for i in range(len(layers) - 1, -1, -1):
        W, b = layers[i]
        gW = dz.T @ acts[i]
        gb = dz.sum(axis=0)
        grads[i] = (gW, gb)
        if i > 0:
            dz = (dz @ W) * gelu_grad(zs[i - 1])
            if bf16:
                dz = bf16_round(dz)
    flat = np.concatenate([np.concatenate([g[0].ravel(), g[1]]) for g in grads])
    return loss, flat


def bf16_round(a):
    """Round float32 values to bfloat16 (nearest even), returned as float64."""
    f = np.asarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    rounding = ((u >> 16) & 1) + 0x7FFF
    r = ((u + rounding) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)
