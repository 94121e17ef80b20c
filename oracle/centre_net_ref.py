"""CPU restatement (numpy) of the centre-proposal network, for gradient checks.

TEST INFRASTRUCTURE ONLY: the checker for the library's CNN kernels (rv_cnn.cu); nothing in the
product imports it.  The network has no counterpart in the reference (RecView leaves the
centre choice to a person looking at a sweep, source/DlgHorizcenter.cpp); it follows the
library's own definition:

    input  X[N, 4, H, W]            bfloat16 values (4 detector rows of a reordered sinogram)
    6 x { conv 3x3 (pad 1) + bias -> ReLU (stored bf16) -> 2x2 average pool (stored bf16) }
         channels 4 -> 32 -> 32 -> 64 -> 64 -> 128 -> 128
    flatten -> FC 128 + bias -> ReLU -> FC 2 + bias -> (mu, s)
    loss   mean_n 0.5 exp(-s) (y - mu)^2 + 0.5 s            (Gaussian negative log-likelihood)

Activations are rounded to bfloat16 where the kernels store them (`bf16=True`); everything else
is float32 (float64 with `bf16=False`, used for finite-difference checks of this file).
"""
from __future__ import annotations

import numpy as np

CHANNELS = (4, 32, 32, 64, 64, 128, 128)
FC_HIDDEN = 128


def bf16(x: np.ndarray) -> np.ndarray:
    """Round float32 values to bfloat16 (nearest, ties to even), returned as float32."""
    a = np.ascontiguousarray(x, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    lsb = (u >> 16) & 1
    r = ((u + 0x7FFF + lsb) >> 16) << 16
    out = r.astype(np.uint32).view(np.float32)
    return np.where(np.isnan(a), a, out)


def init_params(rng: np.random.Generator, H: int, W: int, channels=CHANNELS, hidden=FC_HIDDEN):
    """He-normal weights, zero biases; FC2 starts at (mu, s) = (0, 0)."""
    p = {}
    for l in range(6):
        cin, cout = channels[l], channels[l + 1]
        p[f"w{l}"] = (rng.normal(0, np.sqrt(2.0 / (cin * 9)), (cout, cin, 3, 3))).astype(np.float32)
        p[f"b{l}"] = np.zeros(cout, np.float32)
    nflat = channels[6] * (H >> 6) * (W >> 6)
    p["f0w"] = (rng.normal(0, np.sqrt(2.0 / nflat), (hidden, nflat))).astype(np.float32)
    p["f0b"] = np.zeros(hidden, np.float32)
    p["f1w"] = (rng.normal(0, np.sqrt(1.0 / hidden), (2, hidden)) * 0.1).astype(np.float32)
    p["f1b"] = np.zeros(2, np.float32)
    return p


def _im2col(x):
    n, c, h, w = x.shape
    xp = np.pad(x, ((0, 0), (0, 0), (1, 1), (1, 1)))
    cols = np.empty((n, c, 3, 3, h, w), x.dtype)
    for dy in range(3):
        for dx in range(3):
            cols[:, :, dy, dx] = xp[:, :, dy:dy + h, dx:dx + w]
    return cols.reshape(n, c * 9, h * w)


def conv3x3(x, w, b):
    n, c, h, wd = x.shape
    cols = _im2col(x)                                  # [n, c*9, hw]
    y = np.einsum("ok,nkp->nop", w.reshape(w.shape[0], -1), cols)
    return y.reshape(n, w.shape[0], h, wd) + b[None, :, None, None]


def conv3x3_backward(x, w, dy):
    """dX, dW, db of y = conv3x3(x, w, b)."""
    n, c, h, wd = x.shape
    cols = _im2col(x)
    dyf = dy.reshape(n, dy.shape[1], h * wd)
    dw = np.einsum("nop,nkp->ok", dyf, cols).reshape(w.shape)
    db = dy.sum(axis=(0, 2, 3))
    # dX: full correlation of dy with the flipped kernel
    wf = w[:, :, ::-1, ::-1].transpose(1, 0, 2, 3)      # [c, o, 3, 3]
    dx = conv3x3(dy, wf, np.zeros(c, dy.dtype))
    return dx, dw, db


def avgpool2(x):
    n, c, h, w = x.shape
    return x.reshape(n, c, h // 2, 2, w // 2, 2).mean(axis=(3, 5))


def avgpool2_backward(dy):
    return np.repeat(np.repeat(dy, 2, axis=2), 2, axis=3) * 0.25


def forward(p, x, bf16_store=True):
    """Returns (mu, s, cache)."""
    rnd = bf16 if bf16_store else (lambda a: a)
    dt = np.float32 if bf16_store else np.float64
    a = rnd(np.asarray(x, dt))
    cache = {"in0": a}
    for l in range(6):
        z = conv3x3(a, p[f"w{l}"].astype(dt), p[f"b{l}"].astype(dt))
        r = rnd(np.maximum(z, 0).astype(dt))
        a = rnd(avgpool2(r).astype(dt))
        cache[f"r{l}"] = r
        cache[f"in{l + 1}"] = a
    flat = a.reshape(a.shape[0], -1)
    h = np.maximum(flat @ p["f0w"].astype(dt).T + p["f0b"].astype(dt), 0)
    o = h @ p["f1w"].astype(dt).T + p["f1b"].astype(dt)
    cache["flat"], cache["h"] = flat, h
    return o[:, 0], o[:, 1], cache


def loss_and_grads(p, x, y, bf16_store=True):
    """Gaussian NLL (mean over the batch) and the gradient of every parameter."""
    mu, s, c = forward(p, x, bf16_store)
    dt = mu.dtype
    y = np.asarray(y, dt)
    n = mu.shape[0]
    e = np.exp(-s)
    loss = float(np.mean(0.5 * e * (y - mu) ** 2 + 0.5 * s))
    dmu = (-e * (y - mu)) / n
    ds = (0.5 - 0.5 * e * (y - mu) ** 2) / n
    do = np.stack([dmu, ds], axis=1)
    g = {}
    g["f1w"] = do.T @ c["h"]
    g["f1b"] = do.sum(0)
    dh = (do @ p["f1w"].astype(dt)) * (c["h"] > 0)
    g["f0w"] = dh.T @ c["flat"]
    g["f0b"] = dh.sum(0)
    da = (dh @ p["f0w"].astype(dt)).reshape(c["in6"].shape)
    for l in range(5, -1, -1):
        dr = avgpool2_backward(da) * (c[f"r{l}"] > 0)
        dx, dw, db = conv3x3_backward(c[f"in{l}"], p[f"w{l}"].astype(dt), dr)
        g[f"w{l}"], g[f"b{l}"] = dw, db
        da = dx
    return loss, g, (mu, s)
