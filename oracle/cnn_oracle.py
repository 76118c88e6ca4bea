"""CPU restatement of the learned-correction network. TEST INFRASTRUCTURE ONLY.

The checker for the GPU network kernels in hpc-reading-course_gb300/csrc/cnn.cu
(the network has no counterpart in the reference). Same architecture,
parameter layout and padding: 4 conv3x3 layers, channels (32 -> 32 -> 32 ->
32 -> 16) of which 24 inputs and 3 outputs are real, zero padding at the image
border, ReLU after layers 1-3, mean squared error over the 3 real outputs.

`bf16=True` rounds every tensor the GPU stores in BF16 (inputs, weights,
activations, activation gradients) to BF16 (round to nearest even), so the
remaining difference to the GPU is the FP32 accumulation order.
"""
from __future__ import annotations

import numpy as np

LAYERS = [(32, 32, True), (32, 32, True), (32, 32, True), (32, 16, False)]  # (cin, cout, relu)
IN_REAL, OUT_REAL = 24, 3


def param_count() -> int:
    return sum(co * 9 * ci + co for ci, co, _ in LAYERS)


def unpack(vec):
    """Parameter vector -> [(w (cout, 9, cin), b (cout,)), ...]."""
    out, o = [], 0
    for ci, co, _ in LAYERS:
        w = np.asarray(vec[o:o + co * 9 * ci], dtype=np.float64).reshape(co, 9, ci)
        o += co * 9 * ci
        b = np.asarray(vec[o:o + co], dtype=np.float64)
        o += co
        out.append((w, b))
    return out


def pack(params):
    return np.concatenate([np.concatenate([w.ravel(), b]) for w, b in params])


def round_bf16(a):
    """Round float64 values to the nearest BF16 (ties to even), returned as float64."""
    f = np.asarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def _shift(x, dy, dx):
    """y[b, h, w] = x[b, h + dy, w + dx] with zeros outside."""
    B, H, W, C = x.shape
    y = np.zeros_like(x)
    hs, he = max(0, -dy), min(H, H - dy)
    ws, we = max(0, -dx), min(W, W - dx)
    y[:, hs:he, ws:we] = x[:, hs + dy:he + dy, ws + dx:we + dx]
    return y


def conv3x3(x, w, b=None):
    """y[p][n] = b[n] + sum_{tap, c} x[p + off(tap)][c] w[n][tap][c], tap = (dy+1)*3 + (dx+1)."""
    y = np.zeros(x.shape[:3] + (w.shape[0],))
    for tap in range(9):
        y += _shift(x, tap // 3 - 1, tap % 3 - 1) @ w[:, tap, :].T
    return y if b is None else y + b


def conv3x3_input_grad(d, w):
    """dx[p][c] = sum_{tap, n} d[p - off(tap)][n] w[n][tap][c]."""
    dx = np.zeros(d.shape[:3] + (w.shape[2],))
    for tap in range(9):
        dx += _shift(d, -(tap // 3 - 1), -(tap % 3 - 1)) @ w[:, tap, :]
    return dx


def conv3x3_weight_grad(x, d):
    """dw[n][tap][c] = sum_p d[p][n] x[p + off(tap)][c]."""
    co, ci = d.shape[3], x.shape[3]
    dw = np.zeros((co, 9, ci))
    dm = d.reshape(-1, co)
    for tap in range(9):
        dw[:, tap, :] = dm.T @ _shift(x, tap // 3 - 1, tap % 3 - 1).reshape(-1, ci)
    return dw


def _pad_input(x4):
    x = np.zeros(x4.shape[:3] + (LAYERS[0][0],))
    x[..., :IN_REAL] = x4
    return x


def forward(vec, x4, bf16=True):
    """Network output (B, H, W, 3) and the per-layer inputs (for backward)."""
    rnd = round_bf16 if bf16 else (lambda a: np.asarray(a, dtype=np.float64))
    params = unpack(vec)
    x = rnd(_pad_input(np.asarray(x4, dtype=np.float64)))
    acts = [x]
    for k, ((w, b), (_, _, relu)) in enumerate(zip(params, LAYERS)):
        y = conv3x3(x, rnd(w), b)
        if relu:
            y = np.maximum(y, 0.0)
        if k < len(LAYERS) - 1:
            x = rnd(y)
            acts.append(x)
    return y[..., :OUT_REAL], acts, y


def loss_and_grad(vec, x4, target, bf16=True):
    """Mean squared error over the 3 real outputs and its gradient (parameter layout)."""
    rnd = round_bf16 if bf16 else (lambda a: np.asarray(a, dtype=np.float64))
    params = unpack(vec)
    out3, acts, y = forward(vec, x4, bf16)
    P = out3.shape[0] * out3.shape[1] * out3.shape[2]
    r = out3 - target
    loss = float(np.sum(r * r) / (P * OUT_REAL))
    d = np.zeros_like(y)
    d[..., :OUT_REAL] = 2.0 * r / (P * OUT_REAL)
    d = rnd(d)
    grads = [None] * len(LAYERS)
    for k in range(len(LAYERS) - 1, -1, -1):
        w = rnd(params[k][0])
        grads[k] = (conv3x3_weight_grad(acts[k], d), d.reshape(-1, d.shape[3]).sum(axis=0))
        if k == 0:
            break
        d = rnd(conv3x3_input_grad(d, w))
        d = np.where(acts[k] > 0, d, 0.0)
    return loss, pack(grads)
