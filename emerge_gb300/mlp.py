"""Learned warm start for the frequency sweep.

A small MLP (3 hidden layers of 128, tanh, BF16 weights/activations, FP32
accumulation on the tensor cores; ``emg_mlp_*`` in csrc/emg_mlp.cu) maps
features of (normalised frequency, port) to the coefficients of a column in the
orthonormal basis of the sweep's converged solutions.  It is trained on the GPU
by the project's own forward/backward kernels and Adam, online on the
solutions the sweep has produced, and its prediction only supplies the initial
guess: the Krylov solve still runs to the same FP64 residual tolerance.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib

N_FOURIER = 6


def features(fnorm: np.ndarray, port: np.ndarray, n_ports: int, n_fourier: int = N_FOURIER) -> np.ndarray:
    """[f, sin(k pi f/2), cos(k pi f/2) for k=1..n_fourier, one-hot port] for f in [-1, 1]."""
    f = np.asarray(fnorm, dtype=np.float64)
    cols = [f]
    for k in range(1, n_fourier + 1):
        cols.append(np.sin(k * np.pi * f / 2))
        cols.append(np.cos(k * np.pi * f / 2))
    oh = np.zeros((len(f), n_ports))
    oh[np.arange(len(f)), np.asarray(port, dtype=int)] = 1.0
    return np.concatenate([np.stack(cols, axis=1), oh], axis=1).astype(np.float32)


class MLP:
    """BF16 tensor-core MLP with FP32 master weights (emg_mlp_*)."""

    def __init__(self, in_dim: int, out_dim: int, hidden: int = 128, layers: int = 3, max_batch: int = 1024,
                 seed: int = 0, device="cuda"):
        self.device = torch.device(device)
        self.in_dim, self.out_dim = in_dim, out_dim
        self.max_batch = max_batch
        p = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            _lib.call("emg_mlp_create", in_dim, hidden, layers, out_dim, max_batch, ctypes.c_uint64(seed),
                      ctypes.byref(p))
        self._p = p
        self._lib = _lib.load()
        self.nparam = int(self._lib.emg_mlp_nparam(p))
        self._loss = torch.zeros(1, dtype=torch.float32, device=self.device)

    def __del__(self):
        p = getattr(self, "_p", None)
        if p is not None and p.value:
            try:
                self._lib.emg_mlp_destroy(p)
            except Exception:
                pass
            self._p = None

    @staticmethod
    def _s():
        return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

    def params(self) -> np.ndarray:
        out = np.empty(self.nparam, dtype=np.float32)
        _lib.call("emg_mlp_get_params", self._p, out.ctypes.data_as(ctypes.c_void_p))
        return out

    def set_params(self, w: np.ndarray) -> None:
        w = np.ascontiguousarray(w, dtype=np.float32)
        _lib.call("emg_mlp_set_params", self._p, w.ctypes.data_as(ctypes.c_void_p))

    def forward(self, x: torch.Tensor) -> torch.Tensor:
        x = x.to(self.device, torch.float32).contiguous()
        y = torch.empty((x.shape[0], self.out_dim), dtype=torch.float32, device=self.device)
        _lib.call("emg_mlp_forward", self._p, int(x.shape[0]), ctypes.c_void_p(x.data_ptr()),
                  ctypes.c_void_p(y.data_ptr()), self._s())
        return y

    def step(self, x: torch.Tensor, t: torch.Tensor, lr: float, grads: torch.Tensor | None = None) -> None:
        _lib.call("emg_mlp_train_step", self._p, int(x.shape[0]), ctypes.c_void_p(x.data_ptr()),
                  ctypes.c_void_p(t.data_ptr()), ctypes.c_float(lr), ctypes.c_void_p(self._loss.data_ptr()),
                  ctypes.c_void_p(0 if grads is None else grads.data_ptr()), self._s())

    def loss(self) -> float:
        return float(self._loss.item())

    def gradients(self, x: torch.Tensor, t: torch.Tensor) -> np.ndarray:
        """Loss gradient w.r.t. every parameter (no update)."""
        g = torch.empty(self.nparam, dtype=torch.float32, device=self.device)
        x = x.to(self.device, torch.float32).contiguous()
        t = t.to(self.device, torch.float32).contiguous()
        self.step(x, t, 0.0, g)
        return g.cpu().numpy()

    def fit(self, x: torch.Tensor, t: torch.Tensor, steps: int = 2000, lr: float = 3e-3) -> list[float]:
        x = x.to(self.device, torch.float32).contiguous()
        t = t.to(self.device, torch.float32).contiguous()
        hist = []
        for k in range(steps):
            self.step(x, t, lr * (0.1 if k > 0.8 * steps else 1.0))
            if k % max(1, steps // 10) == 0 or k == steps - 1:
                hist.append(self.loss())
        return hist
