"""Oracle for the warm-start MLP kernels (test infrastructure only).

NumPy FP64 restatement of emerge_gb300's MLP training step, rounding to bf16 at
the same points as the GPU kernels (weights, layer inputs, upstream gradients),
so the GPU forward output and parameter gradients can be checked against it.
Parameter layout: for each linear layer, W (N x K, row-major) then b (N), with
K/N padded to multiples of 16 exactly as emg_mlp_create pads them.
"""
from __future__ import annotations

import numpy as np


def bf16(x: np.ndarray) -> np.ndarray:
    """Round float32 values to bfloat16 (nearest, ties to even), returned as float64."""
    f = np.asarray(x, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    lsb = (u >> 16) & 1
    r = ((u + 0x7FFF + lsb) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def pad16(x: int) -> int:
    return (x + 15) // 16 * 16


def layer_dims(in_dim: int, hidden: int, layers: int, out_dim: int):
    K = [pad16(in_dim)] + [hidden] * layers
    N = [hidden] * layers + [pad16(out_dim)]
    return K, N


def unpack(w: np.ndarray, K, N):
    Ws, bs, off = [], [], 0
    for k, n in zip(K, N):
        Ws.append(w[off:off + n * k].reshape(n, k).astype(np.float64))
        off += n * k
        bs.append(w[off:off + n].astype(np.float64))
        off += n
    return Ws, bs


def forward_backward(w, x, t, in_dim, hidden, layers, out_dim, rounding: bool = True):
    """Returns (output (nb, out_dim), loss, flat gradient) of the GPU training step.

    rounding=False drops the bf16 roundings (and the float32 weights): the exact FP64
    loss and gradient, which a finite-difference test checks the backward formulas on."""
    bf16 = globals()["bf16"] if rounding else (lambda a: np.asarray(a, dtype=np.float64))
    K, N = layer_dims(in_dim, hidden, layers, out_dim)
    Ws, bs = unpack(np.asarray(w, dtype=np.float32 if rounding else np.float64), K, N)
    nb = x.shape[0]
    R = pad16(nb)
    H0 = np.zeros((R, K[0]))
    H0[:nb, :in_dim] = x
    H = [bf16(H0)]
    Z = []
    L = len(K)
    for l in range(L):
        z = H[l] @ bf16(Ws[l]).T + bs[l]
        Z.append(z)
        if l + 1 < L:
            H.append(bf16(np.tanh(z)))
    Y = Z[-1]
    cnt = nb * out_dim
    d = np.zeros_like(Y)
    d[:nb, :out_dim] = Y[:nb, :out_dim] - t
    loss = float(np.sum(d ** 2) / cnt)
    dz_f = 2 * d / cnt
    dz_b = bf16(dz_f)
    grads = []
    for l in range(L - 1, -1, -1):
        gW = dz_b.T @ H[l]
        gb = dz_f[:nb].sum(axis=0)
        grads.append((gW, gb))
        if l > 0:
            dH = dz_b @ bf16(Ws[l])
            th = np.tanh(Z[l - 1])
            dz_f = dH * (1 - th * th)
            dz_b = bf16(dz_f)
    grads = grads[::-1]
    flat = np.concatenate([np.concatenate([gW.ravel(), gb]) for gW, gb in grads])
    return Y[:nb, :out_dim], loss, flat
