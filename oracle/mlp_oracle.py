"""CPU restatement of the warm-start network -- TEST INFRASTRUCTURE ONLY.

The reference has no learned part (its solves start from the uniform state of
source/Initialization.cpp:34-68), so this oracle restates the network the GPU library defines:
features, the forward pass and the backward pass of the mean-squared loss, in numpy, with the
operands rounded to BF16 (round to nearest even) at exactly the points where the GPU kernels
store BF16 (features, pre-activations Z, activations H, the loss gradient dY, every propagated
dZ, the weights), and accumulation in float64 where the GPU accumulates in FP32. It is the
checker of the GPU kernels' outputs and gradients (tests/test_gpu_warmstart.py) and is itself
checked against central finite differences in float64 (tests/test_warmstart_cpu.py). Nothing in
the product imports it.

Parameter layout (as gb_ws_get_params): layer after layer, W[N][K] row-major then b[N];
layers (N, K) = (256, 64), 4 x (256, 256), (16, 256). Outputs 0..5 are used, 6..15 padding.
"""
from __future__ import annotations

import numpy as np

N_IN, HIDDEN, N_OUT, N_USED = 64, 256, 16, 6
LAYERS = [(HIDDEN, N_IN)] + [(HIDDEN, HIDDEN)] * 4 + [(N_OUT, HIDDEN)]


def n_params() -> int:
    return sum(n * k + n for n, k in LAYERS)


def unpack(p):
    """flat parameters -> [(W, b)] (views)"""
    out, o = [], 0
    for n, k in LAYERS:
        w = p[o:o + n * k].reshape(n, k)
        o += n * k
        b = p[o:o + n]
        o += n
        out.append((w, b))
    return out


def bf16(x):
    """float32 -> nearest BF16 (ties to even) -> float32"""
    x = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
    u = x.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return (r & 0xFFFFFFFF).astype(np.uint32).view(np.float32).reshape(x.shape)


def _sig(z):
    return 1.0 / (1.0 + np.exp(-z))


def features(z, r, th, params, norm):
    """the 64 inputs of a cell (float32, before the BF16 rounding): sin / cos(pi 2^f c) of the
    normalised axial position, radius and pitch angle (f = 0..7), the three normalised
    coordinates, the three normalised case parameters, zeros"""
    c = [(np.asarray(v, np.float64) - norm[d]) / (norm[3 + d] - norm[d]) for d, v in enumerate((z, r, th))]
    cols = []
    for d in range(3):
        for f in range(8):
            cols.append(np.sin(np.pi * 2.0 ** f * c[d]))
            cols.append(np.cos(np.pi * 2.0 ** f * c[d]))
    cols += c
    for q in range(3):
        cols.append((np.asarray(params[..., q], np.float64) - norm[6 + q]) / norm[9 + q])
    n = np.broadcast(*cols).shape
    cols = [np.broadcast_to(v, n) for v in cols]
    cols += [np.zeros(n)] * (N_IN - len(cols))
    return np.stack(cols, axis=-1).astype(np.float32)


def forward(p, x, emulate=True):
    """outputs (n x 16) and the stored intermediates; emulate=False: plain float64, no rounding"""
    rd = bf16 if emulate else (lambda v: np.asarray(v, np.float64))
    lay = unpack(np.asarray(p, np.float32 if emulate else np.float64))
    h = rd(x).astype(np.float64)
    X0, Zs, Hs = h, [], []
    for l in range(5):
        w, b = lay[l]
        z = h @ rd(w).astype(np.float64).T + b
        zs = rd(z.astype(np.float32) if emulate else z).astype(np.float64)
        hs = rd((z * _sig(z)).astype(np.float32) if emulate else z * _sig(z)).astype(np.float64)
        Zs.append(zs)
        Hs.append(hs)
        h = hs
    w, b = lay[5]
    y = h @ rd(w).astype(np.float64).T + b
    return y, (X0, Zs, Hs)


def loss_and_grad(p, x, t, emulate=True):
    """mean over samples and the six used outputs of (y - t)^2, and its gradient (flat, the
    parameter layout)"""
    rd = bf16 if emulate else (lambda v: np.asarray(v, np.float64))
    cast = (lambda v: v.astype(np.float32)) if emulate else (lambda v: v)
    y, (X0, Zs, Hs) = forward(p, x, emulate)
    M = x.shape[0]
    e = y[:, :N_USED] - np.asarray(t, np.float64)
    loss = float(np.mean(e * e))
    dY = np.zeros((M, N_OUT))
    dY[:, :N_USED] = rd(cast(2.0 * e / N_USED)).astype(np.float64)
    lay = unpack(np.asarray(p, np.float32 if emulate else np.float64))
    grads = [None] * 6
    grads[5] = (dY.T @ Hs[4] / M, dY.sum(0) / M)
    dH = dY @ rd(lay[5][0]).astype(np.float64)
    for l in range(4, -1, -1):
        z = Zs[l]
        s = _sig(z)
        dZ = rd(cast(dH * (s * (1.0 + z * (1.0 - s))))).astype(np.float64)
        prev = Hs[l - 1] if l > 0 else X0
        grads[l] = (dZ.T @ prev / M, dZ.sum(0) / M)
        if l > 0:
            dH = dZ @ rd(lay[l][0]).astype(np.float64)
    flat = np.concatenate([np.concatenate([g[0].ravel(), g[1].ravel()]) for g in grads])
    return loss, flat
