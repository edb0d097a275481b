"""CPU oracle of the warm-start network (test infrastructure only: used by
tests/ as the checker of odis_mlp_*, never by the product).

A numpy restatement of the same network and loss: layers n_in -> width (GELU)
x depth -> n_mix * n_out, mixed per sample; loss sum_i w_i ||y_i - t_i||^2 / n.
The library rounds every GEMM operand to BF16 (round to nearest even) and
accumulates in FP32; this oracle rounds the same operands at the same points and
accumulates in FP64, so the two agree to FP32-accumulation error (plus the odd
operand whose BF16 rounding flips).  The network has no counterpart in the
reference; its behaviour is pinned by the finite-difference check of this
oracle's own gradient (tests/test_mlp_oracle.py).
"""
from __future__ import annotations

import numpy as np
from scipy.special import erf


def bf16(a) -> np.ndarray:
    """Round to the nearest BF16 value (ties to even), returned as float64."""
    x = np.ascontiguousarray(a, np.float32)
    b = x.view(np.uint32).astype(np.uint64)
    r = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def gelu(z):
    return 0.5 * z * (1.0 + erf(z / np.sqrt(2.0)))


def gelu_grad(z):
    return 0.5 * (1.0 + erf(z / np.sqrt(2.0))) + z * np.exp(-0.5 * z * z) / np.sqrt(2.0 * np.pi)


def dims(n_in, width, depth, n_out, n_mix):
    return [n_in] + [width] * depth + [n_out * max(n_mix, 1)]


def unpack(p, d):
    """Flat parameters -> [(W [out][in], b [out])] in the library's order."""
    out, off = [], 0
    for l in range(len(d) - 1):
        W = p[off:off + d[l + 1] * d[l]].reshape(d[l + 1], d[l]).astype(np.float64)
        off += d[l + 1] * d[l]
        b = p[off:off + d[l + 1]].astype(np.float64)
        off += d[l + 1]
        out.append((W, b))
    return out


def forward(p, d, x, mix=None, n_mix=0, emulate_bf16=True):
    r = bf16 if emulate_bf16 else (lambda a: np.asarray(a, np.float64))
    layers = unpack(p, d)
    h = np.asarray(x, np.float64)
    Z, H = [], [h]
    for l, (W, b) in enumerate(layers):
        z = r(h) @ r(W).T + b
        Z.append(z)
        if l + 1 < len(layers):
            h = gelu(z)
            if emulate_bf16:
                h = h.astype(np.float32).astype(np.float64)
            H.append(h)
    R = Z[-1]
    if n_mix > 0:
        n, n_out = R.shape[0], R.shape[1] // n_mix
        y = np.einsum("ik,iko->io", np.asarray(mix, np.float64), R.reshape(n, n_mix, n_out))
    else:
        y = R
    return y, Z, H


def loss_and_grad(p, d, x, t, mix=None, w=None, n_mix=0, emulate_bf16=True):
    r = bf16 if emulate_bf16 else (lambda a: np.asarray(a, np.float64))
    y, Z, H = forward(p, d, x, mix, n_mix, emulate_bf16)
    n = y.shape[0]
    t = np.asarray(t, np.float64)
    wi = np.ones(n) if w is None else np.asarray(w, np.float64)
    diff = y - t
    loss = float(np.sum(wi[:, None] * diff * diff) / n)
    dy = 2.0 * wi[:, None] * diff / n
    if emulate_bf16:
        dy = dy.astype(np.float32).astype(np.float64)
    if n_mix > 0:
        n_out = dy.shape[1]
        dz = (np.asarray(mix, np.float64)[:, :, None] * dy[:, None, :]).reshape(n, n_mix * n_out)
    else:
        dz = dy
    layers = unpack(p, d)
    grads = []
    for l in range(len(layers) - 1, -1, -1):
        W, _ = layers[l]
        gW = r(dz).T @ r(H[l])
        gb = dz.sum(axis=0)
        grads.append((gW, gb))
        if l > 0:
            dh = r(dz) @ r(W)
            dz = dh * gelu_grad(Z[l - 1])
            if emulate_bf16:
                dz = dz.astype(np.float32).astype(np.float64)
    grads.reverse()
    flat = np.concatenate([np.concatenate([gW.ravel(), gb]) for gW, gb in grads])
    return loss, flat
