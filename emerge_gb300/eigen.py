"""Generalized eigenmodes E x = lambda B x of PEC-restricted systems on the GPU.

Counterpart of the reference's eigen routines: ``SolveRoutine.eig`` →
``SolverARPACK.eig`` (fem/solver.py:348-357, 471-505), ``eigsh(A, k, M=B,
sigma, which)``, and the 3-D cavity code path (fem/physics/edm/emfreq3d.py:
833-848), ``sparse.linalg.eigs(A, k, M=B, sigma=k0^2, which='LM')`` on the
PEC-restricted curl-curl (E) and mass (B) matrices, whose eigenvalues are k0^2.

Method: shift-invert block Arnoldi on Op = (E - sigma B)^-1 B.  The shifted
matrix is factored once with the slab factorization; every application of Op is
an FGMRES solve to an FP64 relative residual of 1e-11 preconditioned by that
factor.  The factor is complex FP64 by default: the shifted cavity operator is
strongly indefinite (the curl-curl null space sits at -sigma B) and its FP32 slab
inverses are too inaccurate to be a useful preconditioner on cube-like cavities
(relative error of one application 0.6-1.5 against 0.1 on waveguides); FP32
(``precision="fp32"``) still converges, with many more inner iterations.  The Krylov basis is orthogonalised
(two classical Gram-Schmidt passes) and the Rayleigh-Ritz problem solved in FP64.
B carries the reference's non-symmetric face-face mass block, so the pencil is
not Hermitian and Arnoldi (not Lanczos) is used, as ``eigs`` does.  Ritz values
theta map back to lambda = sigma + 1/theta; each returned pair is checked by its
FP64 residual ||E x - lambda B x|| / (|lambda| ||B x||).

``which``: "LM" returns the eigenvalues nearest sigma (largest |theta|, the
reference's choice); "LR" the ones just above sigma (largest Re theta): with sigma
below the first nonzero eigenvalue these are the lowest nonzero modes, and the
curl-curl null space (lambda = 0, theta = -1/sigma) stays out of the selection.
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field

import numpy as np
import torch

from .solver import RestrictedSystem, SlabFactor, face_seeds, locality_key


@dataclass
class EigResult:
    eigenvalues: np.ndarray          # lambda = k0^2 (complex; imaginary parts are rounding)
    vectors: torch.Tensor            # (n_restricted, nmodes) complex128, unit 2-norm
    residuals: np.ndarray            # ||E x - lambda B x|| / (|lambda| ||B x||)
    sigma: float
    seconds: float
    info: dict = field(default_factory=dict)

    @property
    def frequencies(self) -> np.ndarray:
        """Resonant frequencies in Hz from k0^2 = lambda."""
        return np.sqrt(np.abs(self.eigenvalues.real)) * 299792458.0 / (2 * np.pi)


def _sync(device) -> None:
    if torch.device(device).type == "cuda":
        torch.cuda.synchronize(device)


class ShiftInvertEigen:
    """Eigenpairs of restricted (E, B) value arrays on a RestrictedSystem.

    Args:
        sysr: the restricted pattern.
        Er, Br: (nnz_r, 1) restricted values of E and B (``RestrictedSystem.form``).
        slab: a SlabFactor of ``sysr`` (its factor is replaced by E - sigma B).
    """

    def __init__(self, sysr: RestrictedSystem, Er: torch.Tensor, Br: torch.Tensor, slab: SlabFactor):
        self.sys, self.Er, self.Br, self.slab = sysr, Er.contiguous(), Br.contiguous(), slab
        self.device = sysr.device
        self.solves = 0
        self.inner_iterations = 0

    def _cm(self, c):
        return torch.zeros(c, dtype=torch.int32, device=self.device)

    def _op(self, A, V, tol):
        """(E - sigma B)^-1 B V by FGMRES on the FP32 slab factor."""
        W = self.sys.spmv(self.Br, V, self._cm(V.shape[1]))
        X, its, res = self.slab.gmres(A, W, self._cm(V.shape[1]), np.zeros(V.shape[1], dtype=np.int32),
                                      restart=40, max_iter=400, tol=tol)
        self.solves += V.shape[1]
        self.inner_iterations += int(its.sum())
        if np.any(res > 100 * tol):
            raise RuntimeError(f"shift-invert solve did not converge (residual {res.max():.2e})")
        return X

    @staticmethod
    def _orth(V, W):
        """W minus its projection on the orthonormal columns of V (two passes)."""
        for _ in range(2):
            W = W - V @ (V.conj().T @ W)
        return W

    def solve(self, nmodes: int, sigma: float, which: str = "LR", block: int = 4, ncv: int | None = None,
              tol: float = 1e-10, max_restarts: int = 30, precision: str = "fp64", seed: int = 0,
              inner_tol: float = 1e-11, refine: int = 0, adapt: bool = False) -> EigResult:
        """nmodes eigenpairs; see the module docstring for ``which``.

        Thick-restarted block Arnoldi: after each Rayleigh-Ritz the wanted Ritz vectors
        (plus a few extra) are kept, orthonormalised, with Op applied to them taken from
        the stored products, and the expansion continues from the block not yet
        expanded.  ``adapt`` (which="LR" only) moves the shift half-way up to a
        converged lowest Ritz value and re-factors; it is off by default because a shift
        close to the first mode makes that mode dominate the Krylov space and slows the
        others."""
        _sync(self.device)
        t0 = time.perf_counter()
        n = self.sys.n
        extra = min(4, max(0, n - nmodes))
        ncv = min(ncv or max(4 * nmodes, 40), n)
        gen = torch.Generator(device="cpu").manual_seed(seed)
        V0 = torch.randn((n, block), generator=gen, dtype=torch.float64).to(self.device).to(torch.complex128)
        lam = res = X = None
        sig = float(sigma)
        factored = None
        shifts = []
        V = torch.linalg.qr(V0)[0].contiguous()    # orthonormal basis; Op known for its first j columns
        OV = []
        j = 0
        for restart in range(max_restarts + 1):
            if factored != sig:
                A = (self.Er - sig * self.Br).contiguous()              # E - sigma B (restricted values)
                self.slab.factor(A, [0], precision, refine)
                factored = sig
                shifts.append(sig)
                if restart > 0:      # a new shift invalidates Op V: restart from the Ritz vectors
                    V = torch.linalg.qr(X)[0].contiguous()
                    OV = []
                    j = 0
            # block Arnoldi on Op = (E - sigma B)^-1 B up to ncv columns
            while j < ncv and j < V.shape[1]:
                Vj = V[:, j:j + block]
                W = self._op(A, Vj.contiguous(), inner_tol)
                OV.append(W)
                j += Vj.shape[1]
                W = self._orth(V, W)
                Qw, Rw = torch.linalg.qr(W)
                good = torch.abs(torch.diagonal(Rw)) > 1e-10 * torch.linalg.norm(W, dim=0).max().clamp_min(1e-300)
                V = torch.cat([V, Qw[:, good]], dim=1).contiguous()
            # Rayleigh-Ritz on span(V[:, :j])
            Vb = V[:, :j]
            OVm = torch.cat(OV, dim=1)[:, :j]
            H = Vb.conj().T @ OVm                                        # (j, j) FP64
            theta, Y = torch.linalg.eig(H)
            th = theta.cpu().numpy()
            order = np.argsort(-np.abs(th)) if which == "LM" else np.argsort(-th.real)
            sel = torch.as_tensor(order[: nmodes + extra], device=self.device)
            Yk = Y[:, sel]
            X = Vb @ Yk
            nrm = torch.linalg.norm(X, dim=0, keepdim=True)
            X = X / nrm
            lam, res, X = self._refine(X, sig + 1.0 / th[order[: nmodes + extra]])
            if np.all(res[:nmodes] <= tol):
                break
            # thick restart: orthonormalised Ritz vectors (Op on them from the stored
            # products, no new solves) followed by the block not yet expanded
            Qk, Rk = torch.linalg.qr(X)
            OVk = torch.linalg.solve_triangular(Rk.T, ((OVm @ Yk) / nrm).T, upper=False).T
            nxt = V[:, j:]
            if nxt.shape[1] == 0:      # the last block was rank deficient: continue from a new random block
                nxt = torch.randn((n, block), generator=gen, dtype=torch.float64).to(self.device).to(torch.complex128)
            nxt = torch.linalg.qr(self._orth(Qk, nxt))[0]
            V = torch.cat([Qk, nxt], dim=1).contiguous()
            OV = [OVk.contiguous()]
            j = Qk.shape[1]
            if adapt and which == "LR":
                lo = int(np.argmin(lam.real))
                l1 = float(lam.real[lo])
                if l1 > sig and res[lo] < 1e-6:
                    nxt_sig = sig + 0.5 * (l1 - sig)
                    if nxt_sig > sig * 1.5:
                        sig = nxt_sig
        _sync(self.device)
        secs = time.perf_counter() - t0
        info = {"restarts": restart, "basis": int(j), "solves": self.solves, "inner_iterations": self.inner_iterations,
                "shifts": shifts, **self.slab.info()}
        lam, res, X = lam[:nmodes], res[:nmodes], X[:, :nmodes]
        o = np.argsort(lam.real)
        return EigResult(lam[o], X[:, torch.as_tensor(o, device=self.device)], res[o], float(sig), secs, info)

    def _refine(self, X, lam):
        """FP64 Rayleigh quotients x^H E x / x^H B x and residuals of unit vectors X."""
        cm = self._cm(X.shape[1])
        EX = self.sys.spmv(self.Er, X.contiguous(), cm)
        BX = self.sys.spmv(self.Br, X.contiguous(), cm)
        num = (X.conj() * EX).sum(dim=0)
        den = (X.conj() * BX).sum(dim=0)
        rq = (num / den).cpu().numpy()
        lam_t = torch.as_tensor(rq, device=self.device)
        R = EX - BX * lam_t[None, :]
        res = (torch.linalg.norm(R, dim=0) / (torch.abs(lam_t) * torch.linalg.norm(BX, dim=0))).cpu().numpy()
        return rq, res, X


class CavityEigen:
    """Eigenmodes of a PEC cavity: volume assembly, restriction, slab plan, shift-invert.

    The slab search starts from the face normal to the cavity's longest side, so
    the slabs are cross-sections of its two shorter sides."""

    def __init__(self, assembler, fieldb, er, ur, bcs):
        plan, E, B = assembler._volume(fieldb, er, ur)
        self.solve_ids = assembler.solve_ids(fieldb, bcs)
        self.sys = RestrictedSystem(plan.indptr, plan.indices[: plan.nnz], plan.nnz, self.solve_ids)
        z = torch.zeros_like(E)
        self.Er = self.sys.form(E, z, [0.0])
        self.Br = self.sys.form(z, B, [-1.0])
        nodes = np.asarray(fieldb.mesh.nodes)
        axis = int(np.argmax(nodes.max(axis=1) - nodes.min(axis=1)))
        self.slab = SlabFactor(self.sys, face_seeds(fieldb, self.solve_ids, axis), locality_key(fieldb, self.solve_ids))
        self.eig = ShiftInvertEigen(self.sys, self.Er, self.Br, self.slab)

    def solve(self, nmodes: int = 10, sigma: float | None = None, **kw) -> EigResult:
        if sigma is None:
            raise ValueError("CavityEigen.solve: give sigma (k0^2 below the wanted modes)")
        return self.eig.solve(nmodes, sigma, **kw)


def box_sigma(dims, eps_max: float, fraction: float = 0.5) -> float:
    """A shift below the first nonzero eigenvalue of a PEC box a x b x c filled with
    permittivity <= eps_max: fraction * (pi^2 (1/a^2 + 1/b^2)) / eps_max with a, b the
    two largest sides (the empty box's lowest k0^2 divided by the largest eps)."""
    s = sorted(dims)[::-1]
    return fraction * np.pi ** 2 * (1 / s[0] ** 2 + 1 / s[1] ** 2) / eps_max


def eig_batch(problems, nmodes: int = 10, assembler=None, sigma_fraction: float = 0.5, **kw) -> list[EigResult]:
    """Lowest nonzero modes of a batch of cavity Problems (uneven sizes), one after
    another on the current stream; each with its own slab plan."""
    from .freq import Assembler
    asm = assembler or Assembler()
    out = []
    for p in problems:
        nodes = np.asarray(p.mesh.nodes)
        dims = nodes.max(axis=1) - nodes.min(axis=1)
        eps_max = float(np.max(np.abs(p.er[0, 0])))
        ce = CavityEigen(asm, p.field, p.er, p.ur, p.bcs)
        r = ce.solve(nmodes, sigma=box_sigma(dims, eps_max, sigma_fraction), which="LR", **kw)
        r.info["n"] = ce.sys.n
        out.append(r)
        del ce
        asm._dev = None          # release this cavity's volume matrices before the next one
    return out
