"""CPU restatement of the warm-start network's kernels.  TEST INFRASTRUCTURE ONLY.

numpy, float64 arithmetic on values rounded to BF16 exactly where the GPU
kernels of ``fft_method_test_gb300/csrc/learned.cu`` round them (layer inputs,
weights, output gradients), so the GPU results differ from these only by
FP32 accumulation order.  Used by tests/test_gpu_learned.py to check the
forward pass, the data and weight gradients and the loss gradient.
"""
from __future__ import annotations

import numpy as np


def bf16(a) -> np.ndarray:
    """Round float values to the nearest BF16 (ties to even), as float64."""
    a = np.asarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def taps(dil: int):
    """(tap index, dz, dy, dx) in the kernels' order, offsets times dil."""
    for t in range(27):
        yield t, (t // 9 - 1) * dil, ((t // 3) % 3 - 1) * dil, (t % 3 - 1) * dil


def shift(x: np.ndarray, dz: int, dy: int, dx: int) -> np.ndarray:
    """x[b, z, y, x_, c] -> x[b, z+dz, y+dy, x_+dx, c] with periodic wrap."""
    return np.roll(x, shift=(-dz, -dy, -dx), axis=(1, 2, 3))


def conv(x: np.ndarray, w: np.ndarray, dil: int, bias=None, relu: bool = False) -> np.ndarray:
    """x [B, nz, ny, nx, cin], w [27, cout, cin] -> y [B, nz, ny, nx, cout]."""
    y = np.zeros(x.shape[:4] + (w.shape[1],))
    for t, dz, dy, dx in taps(dil):
        y += shift(x, dz, dy, dx) @ w[t].T
    if bias is not None:
        y += bias
    return np.maximum(y, 0.0) if relu else y


def conv_data_grad(dy: np.ndarray, w: np.ndarray, dil: int) -> np.ndarray:
    """dx[u] = sum_tap dy[u - off(tap)] @ w[tap]."""
    dx = np.zeros(dy.shape[:4] + (w.shape[2],))
    for t, dz, dyy, dxx in taps(dil):
        dx += shift(dy, -dz, -dyy, -dxx) @ w[t]
    return dx


def conv_weight_grad(dy: np.ndarray, x: np.ndarray, dil: int) -> np.ndarray:
    """dW[tap][o][i] = sum_v dy[v][o] x[v + off(tap)][i]."""
    cout, cin = dy.shape[-1], x.shape[-1]
    dw = np.zeros((27, cout, cin))
    dyf = dy.reshape(-1, cout)
    for t, dz, dyy, dxx in taps(dil):
        dw[t] = dyf.T @ shift(x, dz, dyy, dxx).reshape(-1, cin)
    return dw


def loss_grad(pred: np.ndarray, tgt: np.ndarray, sup: np.ndarray):
    """Per-sample relative squared error of the first 3 channels on the
    support after per-component mean removal, and its gradient.
    pred [B, n, C], tgt [B, n, 3], sup [B, n] bool."""
    B = pred.shape[0]
    loss = np.zeros(B)
    d = np.zeros_like(pred)
    for b in range(B):
        s = sup[b]
        p = pred[b, s, :3]
        r = p - p.mean(axis=0) - tgt[b, s]
        tn = np.sum(tgt[b, s] ** 2)
        loss[b] = np.sum(r ** 2) / tn
        d[b, s, :3] = 2.0 * r / tn
    return loss, d
