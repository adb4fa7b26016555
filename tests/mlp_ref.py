"""f64 numpy restatement of the warm-start network (test reference for the GPU kernels).

Layout and arithmetic follow the library's network: inputs zero-padded to 64, four hidden
layers of 256 with the error-function GELU, one linear output, mean-squared-error loss.
With emulate=True the BF16 roundings of the GPU path are reproduced at the same places
(padded inputs, hidden weights, hidden activations and the backward dz), accumulation in
f64 standing in for the tensor cores' FP32; with emulate=False it is the exact network.
Flat parameter order: W1 [256][64], b1, W2 [256][256], b2, W3, b3, W4, b4, w_out [256], b_out.
"""
from __future__ import annotations

import numpy as np
from scipy.special import erf

WIDTH, HIDDEN, INPAD = 256, 4, 64


def bf16(x) -> np.ndarray:
    """Round to BF16 (nearest, ties to even) through float32."""
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return r.view(np.float32).astype(np.float64)


def f32(x) -> np.ndarray:
    return np.asarray(x, dtype=np.float32).astype(np.float64)


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    W, b, at = [], [], 0
    for layer in range(HIDDEN):
        k = INPAD if layer == 0 else WIDTH
        W.append(p[at:at + WIDTH * k].reshape(WIDTH, k))
        at += WIDTH * k
        b.append(p[at:at + WIDTH])
        at += WIDTH
    w_out = p[at:at + WIDTH]
    b_out = p[at + WIDTH]
    return W, b, w_out, b_out


def gelu(z):
    return 0.5 * z * (1.0 + erf(z / np.sqrt(2.0)))


def gelu_grad(z):
    return 0.5 * (1.0 + erf(z / np.sqrt(2.0))) + z * np.exp(-0.5 * z * z) / np.sqrt(2.0 * np.pi)


def forward(p, x, emulate=True):
    W, b, w_out, b_out = unpack(p)
    x = np.asarray(x, dtype=np.float64)
    X = np.zeros((x.shape[0], INPAD))
    X[:, :x.shape[1]] = x
    if emulate:
        X = bf16(X)
    inputs, zs = [X], []
    h = X
    for layer in range(HIDDEN):
        Wl = bf16(W[layer]) if emulate else W[layer]
        z = h @ Wl.T + (f32(b[layer]) if emulate else b[layer])
        if emulate:
            z = f32(z)
        zs.append(z)
        h = gelu(z)
        if emulate:
            h = bf16(h)
        inputs.append(h)
    y = h @ w_out + b_out
    return y, inputs, zs


def loss_and_grad(p, x, t, emulate=True):
    """(mean squared error, gradient in the flat parameter order)."""
    W, b, w_out, b_out = unpack(p)
    y, inputs, zs = forward(p, x, emulate)
    n = y.shape[0]
    r = y - np.asarray(t, dtype=np.float64)
    loss = float(np.mean(r * r))
    dy = 2.0 * r / n
    h4 = inputs[HIDDEN]
    g_out = h4.T @ dy
    g_bout = dy.sum()
    dz = dy[:, None] * w_out[None, :] * gelu_grad(zs[HIDDEN - 1])
    if emulate:
        dz = bf16(dz)
    gW, gb = [None] * HIDDEN, [None] * HIDDEN
    for layer in range(HIDDEN - 1, -1, -1):
        gW[layer] = dz.T @ inputs[layer]
        gb[layer] = dz.sum(axis=0)
        if layer > 0:
            Wl = bf16(W[layer]) if emulate else W[layer]
            dz = (dz @ Wl) * gelu_grad(zs[layer - 1])
            if emulate:
                dz = bf16(dz)
    parts = []
    for layer in range(HIDDEN):
        parts += [gW[layer].reshape(-1), gb[layer]]
    parts += [g_out, np.array([g_bout])]
    return loss, np.concatenate(parts)


def blocks(n_params=None):
    """Names and slices of the parameter blocks."""
    out, at = [], 0
    for layer in range(HIDDEN):
        k = INPAD if layer == 0 else WIDTH
        out.append((f"W{layer + 1}", slice(at, at + WIDTH * k)))
        at += WIDTH * k
        out.append((f"b{layer + 1}", slice(at, at + WIDTH)))
        at += WIDTH
    out.append(("w_out", slice(at, at + WIDTH)))
    out.append(("b_out", slice(at + WIDTH, at + WIDTH + 1)))
    return out


def init_params(n_in, seed=0):
    """Random parameters of the library's initial scale (input columns >= n_in zero)."""
    rng = np.random.default_rng(seed)
    parts = []
    for layer in range(HIDDEN):
        k = INPAD if layer == 0 else WIDTH
        fan = n_in if layer == 0 else WIDTH
        Wl = rng.uniform(-1, 1, (WIDTH, k)) * np.sqrt(6.0 / fan)
        if layer == 0:
            Wl[:, n_in:] = 0.0
        parts += [Wl.reshape(-1), rng.uniform(-0.1, 0.1, WIDTH)]
    parts += [rng.uniform(-1, 1, WIDTH) * np.sqrt(3.0 / WIDTH), np.array([0.05])]
    return np.concatenate(parts)
