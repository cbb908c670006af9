"""The shift-invert Arnoldi driver (emerge_gb300.eigen) on the CPU: dense stand-ins
for the restricted system and the slab solves, a pencil with a large null space
like curl-curl (E = G^T D G) and a slightly non-symmetric mass matrix like the
reference's.  The lowest nonzero eigenvalues must match LAPACK to 1e-10."""
import numpy as np
import scipy.linalg as sla
import torch

from emerge_gb300.eigen import ShiftInvertEigen


class _Sys:
    device = torch.device("cpu")

    def __init__(self, n):
        self.n = n

    def spmv(self, Av, X, cm, Bv=None):
        Y = Av @ X
        return Y if Bv is None else Bv - Y


class _Slab:
    def factor(self, A, amat, precision, refine):
        self.A = A

    def gmres(self, A, W, cm, cfac, restart, max_iter, tol):
        return torch.linalg.solve(A, W), np.ones(W.shape[1], dtype=int), np.zeros(W.shape[1])

    def info(self):
        return {}


def _pencil(n=300, k=90, seed=0):
    rng = np.random.default_rng(seed)
    G = rng.standard_normal((k, n))
    E = G.T @ np.diag(rng.uniform(1, 50, k)) @ G
    Bm = rng.standard_normal((n, n))
    B = Bm @ Bm.T / n + np.eye(n)
    B[0, 1] += 1e-3
    return E, B


def test_lowest_nonzero_modes_with_null_space():
    E, B = _pencil()
    w = sla.eigvals(E, B)
    w = np.sort(w.real[w.real > 1e-8])
    si = ShiftInvertEigen(_Sys(E.shape[0]), torch.as_tensor(E + 0j), torch.as_tensor(B + 0j), _Slab())
    r = si.solve(6, sigma=0.2 * w[0], which="LR", tol=1e-10)
    assert np.all(r.residuals <= 1e-10)
    assert np.max(np.abs(r.eigenvalues.real - w[:6]) / w[:6]) <= 1e-10
    assert r.info["shifts"] == [0.2 * w[0]]


def test_thick_restart_with_small_basis():
    """A basis of 24 vectors for 6 modes needs several restarts; they must converge."""
    E, B = _pencil()
    w = sla.eigvals(E, B)
    w = np.sort(w.real[w.real > 1e-8])
    si = ShiftInvertEigen(_Sys(E.shape[0]), torch.as_tensor(E + 0j), torch.as_tensor(B + 0j), _Slab())
    r = si.solve(6, sigma=0.2 * w[0], which="LR", tol=1e-10, ncv=24, max_restarts=40)
    assert r.info["restarts"] >= 2
    assert np.max(np.abs(r.eigenvalues.real - w[:6]) / w[:6]) <= 1e-10


def test_nearest_to_sigma():
    E, B = _pencil(seed=1)
    w = sla.eigvals(E, B)
    w = np.sort(w.real[w.real > 1e-8])
    sigma = 0.5 * (w[10] + w[11])
    si = ShiftInvertEigen(_Sys(E.shape[0]), torch.as_tensor(E + 0j), torch.as_tensor(B + 0j), _Slab())
    r = si.solve(4, sigma=sigma, which="LM", tol=1e-10)
    near = w[np.argsort(np.abs(w - sigma))[:4]]
    assert np.max(np.abs(np.sort(r.eigenvalues.real) - np.sort(near)) / near) <= 1e-10
