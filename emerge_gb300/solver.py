"""GPU linear solves of the frequency-domain system.

* ``RestrictedSystem`` — the PEC-restricted pattern ``A[ix_(solve_ids, solve_ids)]``
  (fem/solver.py:434-435) with its ILU(0) schedule, built once per (mesh, PEC set).
* ``GPUSolver`` — drop-in for the ``direct_solver`` slot of the reference
  ``SolveRoutine`` (fem/solver.py:117-131, 405-469): ``solve(A, b, precon,
  reuse_factorization) -> (x, info)``; ILU(0)-preconditioned GMRES in FP64 on the
  GPU, info as in SciPy (0 converged, > 0 iterations without convergence).
* ``FrequencySweep`` — a whole ``frequency_domain`` sweep
  (fem/physics/edm/emfreq3d.py:607-732) with the matrices, the solves and the
  S-parameters resident on the GPU: ``plain`` solves one frequency at a time,
  ``batched`` solves every (frequency, port) column in lockstep, optionally from
  a warm start.
"""
from __future__ import annotations

import ctypes
import time
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _lib
from .bc import C0, is_port


def _vp(t) -> ctypes.c_void_p:
    return ctypes.c_void_p(0 if t is None else t.data_ptr())


def _stream() -> ctypes.c_void_p:
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


class RestrictedSystem:
    """PEC-restricted CSR pattern + ILU(0) structure (emg_rplan)."""

    def __init__(self, indptr: torch.Tensor, indices: torch.Tensor, nnz_full: int, solve_ids: np.ndarray):
        self.device = indptr.device
        self.N = int(indptr.numel() - 1)
        self.nnz_full = int(nnz_full)
        sid = torch.as_tensor(np.ascontiguousarray(solve_ids, dtype=np.int64), device=self.device)
        plan = ctypes.c_void_p()
        _lib.call("emg_rplan_create", self.N, _vp(indptr), _vp(indices), self.nnz_full, int(sid.numel()), _vp(sid),
                  _stream(), ctypes.byref(plan))
        self._plan = plan
        self._lib = _lib.load()
        self.n = int(self._lib.emg_rplan_n(plan))
        self.nnz = int(self._lib.emg_rplan_nnz(plan))
        self.levels = int(self._lib.emg_rplan_levels(plan))
        self.solve_ids = np.asarray(solve_ids, dtype=np.int64)

    def __del__(self):
        p = getattr(self, "_plan", None)
        if p is not None and p.value:
            try:
                self._lib.emg_rplan_destroy(p)
            except Exception:
                pass
            self._plan = None

    def pattern(self):
        """Host copy of the restricted CSR pattern (indptr int64, indices int32)."""
        indptr = np.zeros(self.n + 1, dtype=np.int64)
        indices = np.zeros(max(self.nnz, 1), dtype=np.int32)
        _lib.call("emg_rplan_pattern", self._plan, indptr.ctypes.data_as(ctypes.c_void_p),
                  indices.ctypes.data_as(ctypes.c_void_p))
        return indptr, indices[: self.nnz]

    def form(self, E, B, k2, P=None, gam=None) -> torch.Tensor:
        """Bm restricted matrices (nnz_r, Bm): E - k2[m] B + sum_p gam[p, m] P[p]."""
        k2 = torch.as_tensor(np.ascontiguousarray(k2, dtype=np.float64), device=self.device)
        Bm = int(k2.numel())
        n_ports = 0 if P is None else int(P.shape[0])
        if n_ports:
            gam = torch.as_tensor(np.ascontiguousarray(gam, dtype=np.complex128), device=self.device)
        A = torch.empty((max(self.nnz, 1), Bm), dtype=torch.complex128, device=self.device)
        _lib.call("emg_rplan_form", self._plan, Bm, _vp(E), _vp(B), _vp(k2), n_ports, _vp(P) if n_ports else None,
                  _vp(gam) if n_ports else None, _vp(A), _stream())
        return A

    def ilu0(self, A: torch.Tensor) -> torch.Tensor:
        LU = A.contiguous().clone()
        _lib.call("emg_ilu0", self._plan, int(A.shape[1]), _vp(LU), _stream())
        return LU

    def gather(self, full: torch.Tensor) -> torch.Tensor:
        """full (Bc, N) -> restricted (n, Bc)."""
        Bc = int(full.shape[0])
        out = torch.empty((self.n, Bc), dtype=torch.complex128, device=self.device)
        _lib.call("emg_rplan_gather", self._plan, Bc, _vp(full.contiguous()), _vp(out), _stream())
        return out

    def scatter(self, x: torch.Tensor) -> torch.Tensor:
        """restricted (n, Bc) -> full (Bc, N), zeros on removed DOFs."""
        Bc = int(x.shape[1])
        full = torch.empty((Bc, self.N), dtype=torch.complex128, device=self.device)
        _lib.call("emg_rplan_scatter", self._plan, Bc, _vp(x.contiguous()), _vp(full), _stream())
        return full

    def spmv(self, A, X, cmat, Bv=None) -> torch.Tensor:
        X = X.contiguous()
        A = A.contiguous()
        Bv = None if Bv is None else Bv.contiguous()
        Y = torch.empty(X.shape, dtype=X.dtype, device=X.device)
        _lib.call("emg_spmv", self._plan, int(X.shape[1]), _vp(cmat), int(A.shape[1]), _vp(A), _vp(X),
                  _vp(Bv) if Bv is not None else None, _vp(Y), _stream())
        return Y

    def spmv_family(self, fam, coef, X, Bv=None) -> torch.Tensor:
        """Y = A_c X (or Bv - A_c X) with A_c = sum_a coef[c, a] fam[a] formed on the fly."""
        X = X.contiguous()
        fam = fam.contiguous()
        coef = coef.contiguous()
        Bv = None if Bv is None else Bv.contiguous()
        Y = torch.empty(X.shape, dtype=X.dtype, device=X.device)
        _lib.call("emg_spmv_family", self._plan, int(X.shape[1]), int(fam.shape[0]), _vp(fam), _vp(coef), _vp(X),
                  _vp(Bv) if Bv is not None else None, _vp(Y), _stream())
        return Y

    def gmres(self, A, LU, rhs, cmat, x0=None, restart=150, max_iter=20000, tol=1e-10):
        """Solve column c of rhs (n, Bc) with matrix cmat[c]; returns (x, iters, resid)."""
        Bc = int(rhs.shape[1])
        rhs = rhs.contiguous()
        A = A.contiguous()
        LU = LU.contiguous()
        x = torch.zeros(rhs.shape, dtype=rhs.dtype, device=rhs.device) if x0 is None else x0.contiguous().clone()
        its = torch.zeros(Bc, dtype=torch.int32, device=self.device)
        res = torch.zeros(Bc, dtype=torch.float64, device=self.device)
        _lib.call("emg_gmres", self._plan, Bc, _vp(cmat), int(A.shape[1]), _vp(A), _vp(LU), _vp(rhs.contiguous()),
                  _vp(x), int(restart), int(max_iter), ctypes.c_double(tol), _vp(its), _vp(res), _stream())
        return x, its.cpu().numpy(), res.cpu().numpy()


def dof_positions(field) -> np.ndarray:
    """(3, n_field) position of every DOF: its edge's midpoint or its face's centroid.

    DOF numbering of Nedelec2 (fem/elements/nedelec2.py:46-50): [edges, faces + nE,
    edges + nE + nF, faces + 2 nE + nF]."""
    m = field.mesh
    nodes = np.asarray(m.nodes)
    e_mid = nodes[:, np.asarray(m.edges)].mean(axis=1)
    f_mid = nodes[:, np.asarray(m.tris)].mean(axis=1)
    return np.concatenate([e_mid, f_mid, e_mid, f_mid], axis=1)


def _morton3(q: np.ndarray) -> np.ndarray:
    """Interleaved bits of three 21-bit non-negative integer coordinates (3, n)."""
    def spread(x):
        x = x.astype(np.uint64) & np.uint64(0x1FFFFF)
        x = (x | (x << np.uint64(32))) & np.uint64(0x1F00000000FFFF)
        x = (x | (x << np.uint64(16))) & np.uint64(0x1F0000FF0000FF)
        x = (x | (x << np.uint64(8))) & np.uint64(0x100F00F00F00F00F)
        x = (x | (x << np.uint64(4))) & np.uint64(0x10C30C30C30C30C3)
        x = (x | (x << np.uint64(2))) & np.uint64(0x1249249249249249)
        return x
    return spread(q[0]) | (spread(q[1]) << np.uint64(1)) | (spread(q[2]) << np.uint64(2))


def locality_key(field, solve_ids) -> np.ndarray:
    """Rank of every kept DOF in a Z-order (Morton) walk over its entity's position,
    with the two DOFs of an edge or face next to each other: the order of the DOFs
    inside a slab (see SlabFactor)."""
    sid = np.asarray(solve_ids, dtype=np.int64)
    pos = dof_positions(field)[:, sid]
    lo = pos.min(axis=1, keepdims=True)
    hi = pos.max(axis=1, keepdims=True)
    q = np.round((pos - lo) / np.maximum(hi - lo, 1e-30) * (2 ** 20)).astype(np.int64)
    nE, nF = int(np.asarray(field.mesh.edges).shape[1]), int(np.asarray(field.mesh.tris).shape[1])
    second = sid >= nE + nF
    entity = np.where(second, sid - nE - nF, sid)
    order = np.lexsort((second.astype(np.int64), entity, _morton3(q)))
    key = np.empty(sid.size, dtype=np.int64)
    key[order] = np.arange(sid.size, dtype=np.int64)
    return key


def face_seeds(field, solve_ids, axis: int) -> np.ndarray:
    """Restricted indices of the kept DOFs with the smallest coordinate along ``axis``:
    the start set of a slab search whose slabs are then cross-sections normal to it."""
    pos = dof_positions(field)[axis, np.asarray(solve_ids, dtype=np.int64)]
    lo, hi = float(pos.min()), float(pos.max())
    return np.flatnonzero(pos <= lo + 1e-9 * max(hi - lo, 1e-30)).astype(np.int64)


class SlabFactor:
    """Block-tridiagonal ("slab") factorizations of a RestrictedSystem (emg_slab).

    Breadth-first level sets of the restricted pattern make A block tridiagonal;
    ``factor`` stores the dense inverses of the slab Schur complements of F
    matrices at once, in complex FP32 (``"fp32"``) or FP64 (``"fp64"``).
    """

    def __init__(self, sysr: RestrictedSystem, seeds=None, order_key=None):
        self.sys = sysr
        self._lib = sysr._lib
        h = ctypes.c_void_p()
        sd = np.ascontiguousarray(np.zeros(0) if seeds is None else seeds, dtype=np.int64)
        key = None if order_key is None else np.ascontiguousarray(order_key, dtype=np.int64)
        if key is not None and key.size != sysr.n:
            raise ValueError("SlabFactor: order_key needs one entry per restricted DOF")
        _lib.call("emg_slab_create", sysr._plan, int(sd.size), sd.ctypes.data_as(ctypes.c_void_p) if sd.size else None,
                  key.ctypes.data_as(ctypes.c_void_p) if key is not None else None, _stream(), ctypes.byref(h))
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                self._lib.emg_slab_destroy(h)
            except Exception:
                pass
            self._h = None

    def set_tensor_cores(self, on: bool = True) -> None:
        """Run the wide-group dense products of FP32-factor solves on the tcgen05 tensor
        cores (TF32 products, FP32 accumulation)."""
        _lib.call("emg_slab_set_tensor_cores", self._h, int(bool(on)))

    def set_factor_tensor_cores(self, on: bool = True) -> None:
        """Run the rank-64 updates of FP32 factorizations on the tcgen05 tensor cores
        with split-TF32 products (FP32-equivalent rounding; the default), or on the
        CUDA cores in FP32."""
        _lib.call("emg_slab_set_factor_tensor_cores", self._h, int(bool(on)))

    def set_wide_group(self, min_columns: int) -> None:
        """Column groups of at least ``min_columns`` use the tiled dense products."""
        _lib.call("emg_slab_set_wide_group", self._h, int(min_columns))
        self._wide = int(min_columns)

    def set_max_splits(self, max_splits: int) -> None:
        """Cap on the split-K factor of the tiled dense products."""
        _lib.call("emg_slab_set_max_splits", self._h, int(max_splits))
        self._splits = int(max_splits)

    def autotune(self, columns: int, cfac, repeats: int = 3, candidates=None) -> dict:
        """Pick the product layout for solves of ``columns`` columns with factor map
        ``cfac`` by timing them: the wide-group threshold (tiled vs warp-per-row) and
        the split-K cap.  Keeps the fastest setting; returns {setting: ms} and the
        choice.  Run after ``factor``; the timed solves use random right-hand sides."""
        cand = candidates or [(w, sp) for w in (1, 8, 48, 1 << 30) for sp in (1, 2, 4, 8)]
        cf = np.ascontiguousarray(cfac, dtype=np.int32)
        X = torch.randn((self.sys.n, int(columns)), dtype=torch.complex128, device=self.sys.device)
        times = {}
        for w, sp in cand:
            self.set_wide_group(w)
            self.set_max_splits(sp)
            self.apply(X, cf)                                   # warm-up (allocations)
            torch.cuda.synchronize()
            best = float("inf")
            for _ in range(repeats):
                t0 = time.perf_counter()
                self.apply(X, cf)
                torch.cuda.synchronize()
                best = min(best, time.perf_counter() - t0)
            times[(w, sp)] = 1e3 * best
        choice = min(times, key=times.get)
        self.set_wide_group(choice[0])
        self.set_max_splits(choice[1])
        return {"times_ms": {f"wide={w},splits={sp}": round(t, 3) for (w, sp), t in times.items()},
                "choice": {"wide": choice[0], "max_splits": choice[1]}}

    def info(self) -> dict:
        v = np.zeros(8, dtype=np.int64)
        _lib.call("emg_slab_info", self._h, v.ctypes.data_as(ctypes.c_void_p))
        return {"slabs": int(v[0]), "max_width": int(v[1]), "dense_entries": int(v[2]), "couplings": int(v[3]),
                "factors": int(v[4]), "precision": {0: None, 1: "fp32", 2: "fp64"}[int(v[5])],
                "perturbed_pivots": int(v[6]), "refinements_skipped": int(v[7])}

    def levels(self):
        """(slab boundaries (slabs+1), restricted index of each slab position)."""
        m = self.info()["slabs"]
        off = np.zeros(m + 1, dtype=np.int64)
        perm = np.zeros(self.sys.n, dtype=np.int32)
        _lib.call("emg_slab_levels", self._h, off.ctypes.data_as(ctypes.c_void_p), perm.ctypes.data_as(ctypes.c_void_p))
        return off, perm

    def factor(self, A: torch.Tensor, amat, precision: str = "fp32", refine: int = 0) -> None:
        """Factor the matrices A[:, amat[f]] (A: (nnz_r, Bm) from RestrictedSystem.form);
        ``refine=1``: one Newton-Schulz step on every slab inverse."""
        am = np.ascontiguousarray(amat, dtype=np.int32)
        A = A.contiguous()
        _lib.call("emg_slab_factor", self._h, {"fp32": 1, "fp64": 2}[precision], int(am.size),
                  am.ctypes.data_as(ctypes.c_void_p), int(A.shape[1]), _vp(A), int(refine), _stream())

    def apply(self, X: torch.Tensor, cfac) -> torch.Tensor:
        """A_f^-1 X column by column (X: (n, Bc) complex128), f = cfac[c]."""
        cf = np.ascontiguousarray(cfac, dtype=np.int32)
        X = X.contiguous()
        Y = torch.empty_like(X)
        _lib.call("emg_slab_apply", self._h, int(X.shape[1]), cf.ctypes.data_as(ctypes.c_void_p), _vp(X), _vp(Y),
                  _stream())
        return Y

    def gmres_family(self, fam, coef, rhs, cfac, x0=None, restart=40, max_iter=2000, tol=1e-10):
        """FGMRES with column operators A_c = sum_a coef[c, a] fam[a] formed on the fly
        (fam: (nfam, nnz_r), coef: (Bc, nfam) complex128 device tensors)."""
        sysr = self.sys
        Bc = int(rhs.shape[1])
        cf = np.ascontiguousarray(cfac, dtype=np.int32)
        rhs = rhs.contiguous()
        fam = fam.contiguous()
        coef = coef.contiguous()
        x = torch.zeros(rhs.shape, dtype=rhs.dtype, device=rhs.device) if x0 is None else x0.contiguous().clone()
        its = torch.zeros(Bc, dtype=torch.int32, device=sysr.device)
        res = torch.zeros(Bc, dtype=torch.float64, device=sysr.device)
        _lib.call("emg_gmres_slab_family", sysr._plan, self._h, Bc, int(fam.shape[0]), _vp(fam), _vp(coef),
                  cf.ctypes.data_as(ctypes.c_void_p), _vp(rhs), _vp(x), int(restart), int(max_iter),
                  ctypes.c_double(tol), _vp(its), _vp(res), _stream())
        return x, its.cpu().numpy(), res.cpu().numpy()

    def gmres_mixed(self, A, rhs, cmat, cfac, x0=None, restart=40, max_iter=2000, tol=1e-10, inner_tol=1e-4):
        """Mixed precision (FP32 factors only): FP64 iterative refinement around FGMRES on
        complex FP32 vectors.  Returns (x, inner iterations, residuals, refinement steps)."""
        sysr = self.sys
        Bc = int(rhs.shape[1])
        cf = np.ascontiguousarray(cfac, dtype=np.int32)
        rhs = rhs.contiguous()
        A = A.contiguous()
        x = torch.zeros(rhs.shape, dtype=rhs.dtype, device=rhs.device) if x0 is None else x0.contiguous().clone()
        its = torch.zeros(Bc, dtype=torch.int32, device=sysr.device)
        res = torch.zeros(Bc, dtype=torch.float64, device=sysr.device)
        steps = ctypes.c_int32(0)
        _lib.call("emg_gmres_slab_mixed", sysr._plan, self._h, Bc, _vp(cmat), int(A.shape[1]), _vp(A),
                  cf.ctypes.data_as(ctypes.c_void_p), _vp(rhs), _vp(x), int(restart), int(max_iter),
                  ctypes.c_double(tol), ctypes.c_double(inner_tol), _vp(its), _vp(res), ctypes.byref(steps),
                  _stream())
        return x, its.cpu().numpy(), res.cpu().numpy(), int(steps.value)

    def gmres(self, A, rhs, cmat, cfac, x0=None, restart=40, max_iter=2000, tol=1e-10):
        """FGMRES on column c of rhs with matrix cmat[c], preconditioned by factor cfac[c]."""
        sysr = self.sys
        Bc = int(rhs.shape[1])
        cf = np.ascontiguousarray(cfac, dtype=np.int32)
        rhs = rhs.contiguous()
        A = A.contiguous()
        x = torch.zeros(rhs.shape, dtype=rhs.dtype, device=rhs.device) if x0 is None else x0.contiguous().clone()
        its = torch.zeros(Bc, dtype=torch.int32, device=sysr.device)
        res = torch.zeros(Bc, dtype=torch.float64, device=sysr.device)
        _lib.call("emg_gmres_slab", sysr._plan, self._h, Bc, _vp(cmat), int(A.shape[1]), _vp(A),
                  cf.ctypes.data_as(ctypes.c_void_p), _vp(rhs), _vp(x), int(restart), int(max_iter),
                  ctypes.c_double(tol), _vp(its), _vp(res), _stream())
        return x, its.cpu().numpy(), res.cpu().numpy()


def pattern_key(A) -> tuple:
    """Cache key of a CSR pattern: shape, nnz and a hash of the whole indptr and indices.

    Two patterns with equal row lengths and equal leading columns must not share a
    key (a renumbered mesh of the same structure), so every column index is hashed;
    this is O(nnz) host work, small next to a factorization.
    """
    return (A.shape[0], A.shape[1], int(A.nnz), hash(A.indptr.tobytes()), hash(A.indices.tobytes()))


class GPUSolver:
    """``Solver`` for the reference SolveRoutine (fem/solver.py:117-131) on the GPU.

    ``A`` arrives restricted (CSC/CSR, complex), ``b`` restricted.  ``method``:
    ``"slab"`` (default) — slab factorization in complex FP64 + FGMRES, a direct
    solve like the reference's SuperLU/PARDISO slot; ``"ilu0"`` — level-scheduled
    ILU(0) + GMRES in FP64.  The pattern analysis is cached across calls with the
    same pattern (every frequency of a sweep); with ``reuse_factorization`` the
    previous factors are reused (the second port of the same frequency,
    emfreq3d.py:686-697).
    """

    real_only = False
    req_sorter = False

    def __init__(self, tol: float = 1e-10, restart: int = 150, max_iter: int = 20000, device="cuda",
                 method: str = "slab"):
        if method not in ("slab", "ilu0"):
            raise ValueError(f"GPUSolver: unknown method {method!r}")
        self.own_preconditioner = True
        self.method = method
        self.tol = tol
        self.restart = restart
        self.max_iter = max_iter
        self.device = torch.device(device)
        self._key = None
        self._sys = None
        self._slab = None
        self._A = None
        self._LU = None
        self.last_iterations = 0
        self.last_residual = 0.0

    def __str__(self):
        return "GPUSolver"

    def solve(self, A, b, precon=None, reuse_factorization: bool = False):
        from scipy.sparse import csr_matrix
        A = csr_matrix(A)
        A.sort_indices()
        n = A.shape[0]
        key = pattern_key(A)
        dev = self.device
        if key != self._key:
            indptr = torch.as_tensor(A.indptr.astype(np.int64), device=dev)
            indices = torch.as_tensor(A.indices.astype(np.int32), device=dev)
            self._sys = RestrictedSystem(indptr, indices, A.nnz, np.arange(n))
            self._slab = SlabFactor(self._sys) if self.method == "slab" else None
            self._key = key
            reuse_factorization = False
        sysr = self._sys
        vals = torch.as_tensor(A.data.astype(np.complex128), device=dev)
        zeros = torch.zeros_like(vals)
        if not reuse_factorization or self._A is None:
            self._A = sysr.form(vals, zeros, [0.0])
            if self.method == "slab":
                self._slab.factor(self._A, [0], "fp64")
            else:
                self._LU = sysr.ilu0(self._A)
        rhs = torch.as_tensor(np.asarray(b, dtype=np.complex128), device=dev).reshape(1, n)
        r = sysr.gather(rhs)
        cmat = torch.zeros(1, dtype=torch.int32, device=dev)
        if self.method == "slab":
            x, its, res = self._slab.gmres(self._A, r, cmat, [0], restart=min(self.restart, 40),
                                           max_iter=self.max_iter, tol=self.tol)
        else:
            x, its, res = sysr.gmres(self._A, self._LU, r, cmat, restart=self.restart, max_iter=self.max_iter,
                                     tol=self.tol)
        self.last_iterations = int(its[0])
        self.last_residual = float(res[0])
        info = 0 if res[0] <= self.tol * 10 else int(its[0])
        return sysr.scatter(x)[0].cpu().numpy(), info


# ------------------------------------------------------------------ sweep ---
@dataclass
class SweepResult:
    freqs: np.ndarray
    S: np.ndarray                     # (nf, np, np) complex
    iterations: np.ndarray            # (nf, np)
    residuals: np.ndarray             # (nf, np) explicit relative residuals
    seconds: float                    # wall time of the solve phase
    solutions: torch.Tensor | None = None   # (n, nf*np) restricted solutions (device)
    info: dict = field(default_factory=dict)


class FrequencySweep:
    """Frequency sweep of ``Electrodynamics3D.frequency_domain`` on the GPU.

    Args:
        assembler: an ``emerge_gb300.freq.Assembler`` (volume E, B cached on it).
        field, er, ur, bcs: as for ``Assembler.assemble_freq_matrix``.

    Port matrices are linear in gamma (Robin blocks, fem/mth/tri.py:630,694), so
    A(k) = E - k^2 B + sum_p gamma_p(k) P_p with unit matrices P_p built once;
    port right-hand sides are linear in beta (U_inc = -2j beta E_mode,
    fem/bc.py:588-589), b_p(k) = -2j beta_p(k) u_p with u_p = int N . E_mode.
    S-parameters use the same quadrature as fem/mth/sparam.py:102-139:
    S_ij = (-x_j . u_i - delta_ij P_i) / P_i, P_i = int |E_mode_i|^2, since the
    forcing entries are u_i = -int N . E_mode_i.
    """

    def __init__(self, assembler, field, er, ur, bcs):
        self.asm = assembler
        self.field = field
        self.bcs = bcs
        self.ports = sorted([bc for bc in bcs if is_port(bc)], key=lambda b: b.port_number)
        dev = assembler.device
        self.device = dev
        plan, E, B = assembler._volume(field, er, ur)
        self.plan, self.E, self.B = plan, E, B
        N = plan.n_field
        # unit port matrices (gamma = 1) and unit forcing vectors (U_inc = E_mode)
        unit_bcs = []
        for bc in bcs:
            unit_bcs.append(_UnitRobin(bc) if hasattr(bc, "get_gamma") and hasattr(bc, "_include_stiff") else bc)
        robin = [u for u in unit_bcs if isinstance(u, _UnitRobin)]
        self.robin = robin
        sysd = assembler.device_system(field, er, ur, unit_bcs, frequency=C0 / (2 * np.pi))   # k0 = 1
        # per Robin BC: its unit matrix alone = K(unit only) - (E - B); build each separately
        P = torch.zeros((len(robin), plan.nnz), dtype=torch.complex128, device=dev)
        for i, u in enumerate(robin):
            solo = [b for b in unit_bcs if not isinstance(b, _UnitRobin)] + [u]
            s1 = assembler.device_system(field, er, ur, solo, frequency=C0 / (2 * np.pi))
            P[i] = s1.K - (E - B)
        self.P = P
        self.u = {bc.port_number: sysd.port_vectors[bc.port_number] for bc in self.ports}
        self.solve_ids = sysd.solve_ids
        self.sys = RestrictedSystem(plan.indptr, plan.indices[: plan.nnz], plan.nnz, self.solve_ids)
        self.u_r = self.sys.gather(torch.stack([self.u[bc.port_number] for bc in self.ports]))   # (n, np)
        # per waveport triangle, the material weight of its mode integrals (emfreq3d.py:767-778);
        # the S-parameter functionals u_w carry it, the forcing u_r does not
        self.sconst = [None if _is_lumped(bc) else _port_const(field, bc, er, ur) for bc in self.ports]
        self.u_w = self._weighted_functionals(assembler, field, er, ur, unit_bcs)
        self.Pmode = np.array([_mode_power(field, bc, c) for bc, c in zip(self.ports, self.sconst)])
        # forcing amplitude per unit port mode: U_inc = -2j beta amp E_mode (1 for waveports,
        # whose mode carries its amplitude; V/h * 376.7303/Zs for lumped ports)
        self.amp = np.array([_lumped_amp(bc) if _is_lumped(bc) else 1.0 for bc in self.ports])
        self._vfun = self._voltage_functionals()

    def _weighted_functionals(self, assembler, field, er, ur, unit_bcs):
        """(n, np) restricted functionals G_i(x) = -u_w,i . x = int const E . E_mode_i.

        A port whose faces carry one material weight c gets c * u_i; a port with
        mixed fills gets its forcing vector assembled again with U_inc scaled by
        each triangle's weight."""
        cols = []
        for i, bc in enumerate(self.ports):
            c = self.sconst[i]
            if c is None or len(c) == 0 or np.all(c == c[0]):
                w = 1.0 if c is None or len(c) == 0 else complex(c[0])
                cols.append(self.u_r[:, i] * w)
                continue
            solo = [b for b in unit_bcs if not isinstance(b, _UnitRobin) or b.bc is bc]
            sw = assembler.device_system(field, er, ur, solo, frequency=C0 / (2 * np.pi),
                                         force_weights={bc.port_number: c})
            cols.append(self.sys.gather(sw.port_vectors[bc.port_number].reshape(1, -1))[0])
        return torch.stack(cols, dim=1)

    def _voltage_functionals(self):
        """Per lumped port, its line voltage sum_i E(mid_i) . dl_i as a sparse functional of
        the restricted solution (fem/physics/edm/emfreq3d.py:752-757), the field searched
        over the tets that touch a port face, last containing tet winning
        (all_port_tets, emfreq3d.py:648-653)."""
        from .field import line_weights
        out = {}
        lumped = [i for i, bc in enumerate(self.ports) if _is_lumped(bc)]
        if not lumped:
            return out
        m = self.field.mesh
        verts = np.unique(np.concatenate([np.asarray(m.tris)[:, np.asarray(m.get_triangles(bc.tags), dtype=np.int64)]
                                          .ravel() for bc in self.ports]))
        hit = np.isin(np.asarray(m.tets), verts).any(axis=0)
        port_tets = np.flatnonzero(hit)
        N = self.plan.n_field
        full2r = torch.full((N,), -1, dtype=torch.int64, device=self.device)
        full2r[torch.as_tensor(self.solve_ids, device=self.device)] = torch.arange(self.sys.n, device=self.device)
        for i in lumped:
            mid, step = _lumped_line(self.ports[i], m)
            dofs, w = line_weights(self.field, mid, step, tetids=port_tets, device=self.device)
            dofs, w = dofs.reshape(-1), w.reshape(-1)
            r = torch.where(dofs >= 0, full2r[dofs.clamp_min(0)], torch.full_like(dofs, -1))
            keep = r >= 0                      # PEC DOFs hold zero
            out[i] = (r[keep], w[keep].to(torch.complex128))
        return out

    def _coeffs(self, freqs):
        k0 = 2 * np.pi * np.asarray(freqs, dtype=float) / C0
        gam = np.array([[complex(u.bc.get_gamma(k)) for k in k0] for u in self.robin]).reshape(len(self.robin), len(k0))
        beta = np.array([[complex(bc.get_beta(k)) for k in k0] for bc in self.ports])     # (np, nf)
        return k0, gam, beta

    def _rhs(self, beta):
        """(n, nf*np) restricted right-hand sides, column f*np + p."""
        nf = beta.shape[1]
        npo = len(self.ports)
        scale = torch.as_tensor((-2j * beta.T * self.amp[None, :]).reshape(-1), device=self.device)  # (nf*np)
        cols = self.u_r[:, torch.arange(npo, device=self.device).repeat(nf)]                    # (n, nf*np)
        return cols * scale[None, :]

    def _sparams(self, X, nf, beta, k0):
        """S[f, i, j] = pfield_i / pmode_j for the column of frequency f driven at port j
        (fem/physics/edm/emfreq3d.py:690-766).

        Waveports (fem/mth/sparam.py:72-139): int E_c . E_mode_i = -x_c . u_i (the forcing
        of fem/mth/tri.py:668-693 is -int N . U_inc, so u_i = -int N . E_mode_i; E_mode real),
        pfield = (int E . E_mode - [i = j] P_i) / (2 Z_i), pmode = P_j / (2 Z_j).
        Lumped ports (emfreq3d.py:752-766): V = line voltage, pfield = sqrt((V - [i = j] V0)^2
        / (2 Z0)), pmode = sqrt(V0^2 / (2 Z0)), principal square roots as the reference."""
        npo = len(self.ports)
        G = -(self.u_w.T @ X).cpu().numpy()                                                      # (np, nf*np)
        V = {i: (w[:, None] * X[r]).sum(dim=0).cpu().numpy() for i, (r, w) in self._vfun.items()}
        S = np.zeros((nf, npo, npo), dtype=np.complex128)
        for f in range(nf):
            for j in range(npo):
                bj = self.ports[j]
                if _is_lumped(bj):
                    pm = np.sqrt(complex(bj.voltage) ** 2 / (2 * bj.Z0))
                else:
                    pm = self.Pmode[j] / (2 * _zmode(bj, k0[f]))
                for i in range(npo):
                    bi = self.ports[i]
                    c = f * npo + j
                    if _is_lumped(bi):
                        bv = V[i][c] - (bi.voltage if i == j else 0.0)
                        pf = np.sqrt(bv ** 2 / (2 * bi.Z0))
                    else:
                        pf = (G[i, c] - (self.Pmode[i] if i == j else 0.0)) / (2 * _zmode(bi, k0[f]))
                    S[f, i, j] = pf / pm
        return S

    def slab(self, seeds: str = "port") -> SlabFactor:
        """The slab structure of the restricted system (built on first use).

        ``seeds="port"``: the search starts from the DOFs on the first port's face, so
        the slabs are cross-sections of a guide.  ``seeds="axis"``: it starts from the
        DOFs of least coordinate along the domain's longest axis, so the slabs are
        planar cross-sections of the whole domain, which suits open structures fed by a
        small port (the port seeds would grow shells around it)."""
        if getattr(self, "_slab", None) is None:
            sd = None
            if seeds == "axis":
                ext = np.ptp(np.asarray(self.field.mesh.nodes), axis=1)
                sd = face_seeds(self.field, self.solve_ids, int(np.argmax(ext)))
            elif self.ports:
                u = self.u[self.ports[0].port_number].abs().cpu().numpy()
                on_port = np.flatnonzero(u[self.solve_ids] > 0)
                sd = on_port if on_port.size else None
            seeds = sd
            self._slab = SlabFactor(self.sys, seeds, locality_key(self.field, self.solve_ids))
            self._slab_key = None
        return self._slab

    def factor_anchors(self, anchors, precision: str = "fp32", refine: int = 0) -> float:
        """Slab factorizations of A(k) at the anchor frequencies (cached); returns seconds."""
        anchors = np.asarray(anchors, dtype=float)
        key = (tuple(anchors.tolist()), precision, refine)
        sl = self.slab()
        if self._slab_key == key:
            return 0.0
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        k0, gam, _ = self._coeffs(anchors)
        A = self.sys.form(self.E, self.B, k0 ** 2, self.P, gam)
        sl.factor(A, np.arange(len(anchors)), precision, refine)
        del A
        torch.cuda.synchronize()
        self._slab_key = key
        return time.perf_counter() - t0

    def autotune(self, freqs, n_anchor: int = 8, chunk: int | None = None, precision: str = "fp32") -> dict:
        """Tune the slab products (``SlabFactor.autotune``) for this sweep's column
        pattern: the anchors' factors and one chunk of (frequency, port) columns."""
        freqs = np.asarray(freqs, dtype=float)
        anchors = self.default_anchors(freqs, n_anchor)
        self.factor_anchors(anchors, precision)
        nf, npo = len(freqs), len(self.ports)
        c = min(nf, chunk or nf)
        near = np.argmin(np.abs(freqs[:c, None] - anchors[None, :]), axis=1)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out = self.slab().autotune(c * npo, np.repeat(near, npo),
                                   candidates=[(w, sp) for w in (8, 1 << 30) for sp in (1, 4, 8)])
        out["seconds"] = time.perf_counter() - t0
        return out

    @staticmethod
    def default_anchors(freqs, n_anchor: int) -> np.ndarray:
        """Centres of n_anchor equal sub-bands of [min(freqs), max(freqs)]."""
        lo, hi = float(np.min(freqs)), float(np.max(freqs))
        n_anchor = max(1, int(n_anchor))
        return lo + (np.arange(n_anchor) + 0.5) * (hi - lo) / n_anchor

    def run_anchored(self, freqs, n_anchor: int = 4, anchors=None, precision: str = "fp32", tol: float = 1e-10,
                     restart: int = 40, max_iter: int = 2000, x0: torch.Tensor | None = None,
                     chunk: int | None = None, refine: int = 0, operators: str = "stored",
                     inner: str = "fp64") -> SweepResult:
        """Batched FGMRES sweep preconditioned by slab factorizations at anchor frequencies.

        Every (frequency, port) column runs FP64 FGMRES to ``tol`` on its own A(k),
        preconditioned by the factor of the nearest anchor; with ``precision="fp32"``
        the factors and their solves are complex FP32 (mixed precision: FP32 inner,
        FP64 residuals and updates).  ``operators``: "stored" forms A(k) for every
        frequency of a chunk (16 nnz_r bytes per frequency; one complex FP64 MAC per
        nonzero and column in the products); "family" keeps only E, B and the port
        matrices and forms A(k) inside every product (2 + n_ports MACs per nonzero
        and column: slower on GB300's FP64 pipes, for when memory is short).
        ``inner="fp32"`` (FP32 factors, stored operators): FP64 iterative refinement
        around FGMRES on complex FP32 vectors and an FP32 copy of A(k); the
        iteration counts are then inner iterations summed over refinement steps."""
        freqs = np.asarray(freqs, dtype=float)
        nf, npo = len(freqs), len(self.ports)
        anchors = self.default_anchors(freqs, n_anchor) if anchors is None else np.asarray(anchors, dtype=float)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        t_fac = self.factor_anchors(anchors, precision, refine)
        k0, gam, beta = self._coeffs(freqs)
        near = np.argmin(np.abs(freqs[:, None] - anchors[None, :]), axis=1)
        sysr, sl = self.sys, self.slab()
        X = torch.zeros((sysr.n, nf * npo), dtype=torch.complex128, device=self.device)
        its = np.zeros(nf * npo, dtype=np.int64)
        res = np.zeros(nf * npo)
        chunk = chunk or nf
        steps = 0
        fam = self.family() if operators == "family" else None
        # column coefficients of A(k) = E - k^2 B + sum_p gamma_p P_p, one row per frequency
        cf = np.zeros((nf, 2 + gam.shape[0]), dtype=np.complex128)
        cf[:, 0] = 1.0
        cf[:, 1] = -k0 ** 2
        cf[:, 2:] = gam.T
        for f0 in range(0, nf, chunk):
            f1 = min(nf, f0 + chunk)
            rhs = self._rhs(beta[:, f0:f1])
            cfac = np.repeat(near[f0:f1], npo)
            xin = None if x0 is None else x0[:, f0 * npo:f1 * npo]
            if operators == "family":
                coef = torch.as_tensor(np.repeat(cf[f0:f1], npo, axis=0), device=self.device)
                x, it, rs = sl.gmres_family(fam, coef, rhs, cfac, x0=xin, restart=restart, max_iter=max_iter, tol=tol)
            else:
                A = sysr.form(self.E, self.B, k0[f0:f1] ** 2, self.P, gam[:, f0:f1])
                cmat = torch.arange(f1 - f0, dtype=torch.int32, device=self.device).repeat_interleave(npo)
                if inner == "fp32" and precision == "fp32":
                    x, it, rs, nsteps = sl.gmres_mixed(A, rhs, cmat, cfac, x0=xin, restart=restart,
                                                       max_iter=max_iter, tol=tol)
                    steps = max(steps, nsteps)
                else:
                    x, it, rs = sl.gmres(A, rhs, cmat, cfac, x0=xin, restart=restart, max_iter=max_iter, tol=tol)
                del A
            X[:, f0 * npo:f1 * npo] = x
            its[f0 * npo:f1 * npo] = it
            res[f0 * npo:f1 * npo] = rs
        # S-parameter extraction is part of the solve phase (it ends with a device-to-host copy)
        S = self._sparams(X, nf, beta, k0)
        secs = time.perf_counter() - t0
        info = {"anchors": anchors, "precision": precision, "refine": refine, "inner": inner,
                "refinement_steps": steps, "factor_seconds": t_fac, **sl.info()}
        return SweepResult(freqs, S, its.reshape(nf, npo), res.reshape(nf, npo), secs, X, info)

    def run(self, freqs, method: str = "batched", tol: float = 1e-10, restart: int = 150, max_iter: int = 20000,
            x0: torch.Tensor | None = None, chunk: int | None = None, precond: str = "ilu0") -> SweepResult:
        """``plain``: one frequency at a time, its own preconditioner and solve (both
        ports together); ``batched``: every column in lockstep (ILU(0)).  ``precond``
        of the plain method: ``"ilu0"`` (level-scheduled ILU(0) + GMRES) or
        ``"slab64"`` / ``"slab32"`` (slab factorization of that frequency in complex
        FP64 / FP32 + FGMRES: a direct solve with FP64 refinement)."""
        freqs = np.asarray(freqs, dtype=float)
        nf, npo = len(freqs), len(self.ports)
        k0, gam, beta = self._coeffs(freqs)
        sysr = self.sys
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        X = torch.zeros((sysr.n, nf * npo), dtype=torch.complex128, device=self.device)
        its = np.zeros(nf * npo, dtype=np.int64)
        res = np.zeros(nf * npo)
        if method == "plain":
            for f in range(nf):
                A = sysr.form(self.E, self.B, [k0[f] ** 2], self.P, gam[:, f:f + 1])
                rhs = self._rhs(beta[:, f:f + 1])
                cmat = torch.zeros(npo, dtype=torch.int32, device=self.device)
                if precond == "ilu0":
                    LU = sysr.ilu0(A)
                    x, it, rs = sysr.gmres(A, LU, rhs, cmat, restart=restart, max_iter=max_iter, tol=tol)
                else:
                    sl = self.slab()
                    sl.factor(A, [0], {"slab64": "fp64", "slab32": "fp32"}[precond])
                    self._slab_key = None
                    x, it, rs = sl.gmres(A, rhs, cmat, np.zeros(npo, dtype=np.int32), restart=min(restart, 40),
                                         max_iter=max_iter, tol=tol)
                X[:, f * npo:(f + 1) * npo] = x
                its[f * npo:(f + 1) * npo] = it
                res[f * npo:(f + 1) * npo] = rs
        else:
            chunk = chunk or nf
            for f0 in range(0, nf, chunk):
                f1 = min(nf, f0 + chunk)
                A = sysr.form(self.E, self.B, k0[f0:f1] ** 2, self.P, gam[:, f0:f1])
                LU = sysr.ilu0(A)
                rhs = self._rhs(beta[:, f0:f1])
                cmat = torch.arange(f1 - f0, dtype=torch.int32, device=self.device).repeat_interleave(npo)
                xin = None if x0 is None else x0[:, f0 * npo:f1 * npo]
                x, it, rs = sysr.gmres(A, LU, rhs, cmat, x0=xin, restart=restart, max_iter=max_iter, tol=tol)
                X[:, f0 * npo:f1 * npo] = x
                its[f0 * npo:f1 * npo] = it
                res[f0 * npo:f1 * npo] = rs
        S = self._sparams(X, nf, beta, k0)
        secs = time.perf_counter() - t0
        return SweepResult(freqs, S, its.reshape(nf, npo), res.reshape(nf, npo), secs, X)


    def family(self) -> torch.Tensor:
        """(2 + n_robin, nnz_r) restricted values of E, B and the unit port matrices: the
        matrix family whose combination (1, -k^2, gamma_1(k), ...) is A(k)."""
        if getattr(self, "_fam", None) is None:
            Er, Br, Pr = self._restricted_parts()
            self._fam = torch.stack([Er[:, 0], Br[:, 0]] + [P[:, 0] for P in Pr]).contiguous()
        return self._fam

    # ------------------------------------------------------------ warm start ---
    def _restricted_parts(self):
        """Restricted E, B and unit port matrices as single-matrix value arrays (nnz_r, 1)."""
        if getattr(self, "_parts", None) is None:
            z = torch.zeros_like(self.E)
            Er = self.sys.form(self.E, z, [0.0])
            Br = self.sys.form(z, self.B, [-1.0])
            Pr = []
            for i in range(self.P.shape[0]):
                g = np.zeros((self.P.shape[0], 1), dtype=np.complex128)
                g[i, 0] = 1.0
                Pr.append(self.sys.form(z, z, [0.0], self.P, g))
            self._parts = (Er, Br, Pr)
        return self._parts

    def _reduced(self, Xs: torch.Tensor):
        """Orthonormal basis Q of span(Xs) and the Gram blocks of the reduced system.

        With Z_a = (E, B, P_1, ...) Q and alpha(k) = (1, -k^2, gamma_1(k), ...),
        A(k) Q = sum_a alpha_a Z_a, so min ||A(k) Q y - b(k)|| only needs the small
        blocks Z_a^H Z_b and Z_a^H u_p, computed once: returns (Q, Gab, Hu)."""
        Q, _ = torch.linalg.qr(Xs)                       # orthonormal basis (n, r)
        Q = Q.contiguous()                               # LAPACK order is column-major
        Er, Br, Pr = self._restricted_parts()
        r = Q.shape[1]
        cm = torch.zeros(r, dtype=torch.int32, device=self.device)
        Zs = [self.sys.spmv(Er, Q, cm), self.sys.spmv(Br, Q, cm)] + [self.sys.spmv(Pi, Q, cm) for Pi in Pr]
        Zc = torch.stack(Zs)                              # (na, n, r)
        Gab = torch.einsum("ani,bnj->abij", Zc.conj(), Zc)               # (na, na, r, r)
        Hu = torch.einsum("ani,np->api", Zc.conj(), self.u_r)           # (na, np, r)
        return Q, Gab, Hu

    def _min_res_coeffs(self, Gab, Hu, freqs) -> torch.Tensor:
        """Coefficients y(f, p) (nf, np, r) of min ||A(k) Q y - b_p(k)|| (normal equations)."""
        freqs = np.asarray(freqs, dtype=float)
        k0, gam, beta = self._coeffs(freqs)
        nf, npo, na, r = len(freqs), len(self.ports), Gab.shape[0], Gab.shape[2]
        alpha = np.zeros((nf, na), dtype=np.complex128)
        alpha[:, 0] = 1.0
        alpha[:, 1] = -k0 ** 2
        alpha[:, 2:] = gam.T
        al = torch.as_tensor(alpha, device=self.device)                 # (nf, na)
        G = torch.einsum("fa,fb,abij->fij", al.conj(), al, Gab)          # (nf, r, r)
        h = torch.einsum("fa,api->fpi", al.conj(), Hu)                   # (nf, np, r)
        bscale = torch.as_tensor(-2j * beta.T * self.amp[None, :], device=self.device)   # (nf, np)
        h = h * bscale[:, :, None]
        # ridge-free solve; G is Hermitian positive definite on a full-rank basis
        return torch.linalg.solve(G[:, None, :, :].expand(nf, npo, r, r), h[..., None])[..., 0]

    def project(self, Xs: torch.Tensor, freqs, ports=None) -> torch.Tensor:
        """Minimal-residual initial guesses in span(Xs) for every (frequency, port)
        column (the reduced system of ``_reduced``).  Returns X0 (n, nf*np)."""
        Q, Gab, Hu = self._reduced(Xs)
        y = self._min_res_coeffs(Gab, Hu, freqs)                          # (nf, np, r)
        return Q @ y.reshape(-1, Q.shape[1]).T                            # (n, nf*np)

    def mlp_guess(self, Xs: torch.Tensor, train_freqs, freqs, steps: int = 1500, seed: int = 0,
                  target: str = "solutions", n_dense: int = 256, n_fourier: int | None = None):
        """Initial guesses from the warm-start MLP trained on the converged columns Xs.

        The network maps (normalised frequency, port) to coefficients in the orthonormal
        basis Q of span(Xs) (real and imaginary parts, each standardised).  Targets:
          "solutions": the coefficients of the training columns themselves (the
                       network interpolates between the training frequencies);
          "minres":    the minimal-residual coefficients of the reduced system at
                       ``n_dense`` frequencies spread over the band (offset from the
                       sweep's own), computed from the same converged columns, so the
                       network learns the reduced solution between the training
                       points and the guess approaches the projection's.
        ``n_fourier``: Fourier features of the frequency (default 6 for "solutions",
        16 for "minres", whose targets resolve the passband's resonances).
        Returns (X0, final training loss)."""
        from .mlp import MLP, features
        nfo = n_fourier if n_fourier is not None else (16 if target == "minres" else 6)
        npo = len(self.ports)
        f_lo, f_hi = float(np.min(freqs)), float(np.max(freqs))
        fn = lambda f: 2 * (np.asarray(f, dtype=float) - f_lo) / max(f_hi - f_lo, 1e-30) - 1   # noqa: E731
        if target == "minres":
            Q, Gab, Hu = self._reduced(Xs)
            fd = f_lo + (np.arange(n_dense) + 0.5) * (f_hi - f_lo) / n_dense
            Y = self._min_res_coeffs(Gab, Hu, fd).reshape(n_dense * npo, -1)   # (nd*np, r)
            tf = fd
        elif target == "solutions":
            Q, _ = torch.linalg.qr(Xs)
            Q = Q.contiguous()
            Y = (Q.conj().T @ Xs).T                                       # (nt*np, r) complex
            tf = np.asarray(train_freqs, dtype=float)
        else:
            raise ValueError(f"mlp_guess: unknown target {target!r}")
        T = torch.cat([Y.real, Y.imag], dim=1)
        # each output standardised on its own: the basis coefficients span orders of
        # magnitude, and one common scale would leave the small ones unlearned
        mu = T.mean(dim=0, keepdim=True)
        scale = T.std(dim=0, keepdim=True).clamp_min(1e-30 + 1e-12 * T.abs().max().item())
        T = ((T - mu) / scale).to(torch.float32).contiguous()
        xt = features(np.repeat(fn(tf), npo), np.tile(np.arange(npo), len(tf)), npo, nfo)
        fq = np.asarray(freqs, dtype=float)
        net = MLP(xt.shape[1], T.shape[1], max_batch=max(64, len(xt), len(fq) * npo), seed=seed, device=self.device)
        hist = net.fit(torch.as_tensor(xt), T, steps=steps, lr=3e-3)
        xa = features(np.repeat(fn(fq), npo), np.tile(np.arange(npo), len(fq)), npo, nfo)
        P = net.forward(torch.as_tensor(xa)).to(torch.float64) * scale + mu    # (nf*np, 2r)
        r = Q.shape[1]
        yc = torch.complex(P[:, :r], P[:, r:])
        return (Q @ yc.T).contiguous(), hist[-1]

    def _merge(self, freqs, idx_a, res_a: SweepResult, idx_b, res_b: SweepResult) -> SweepResult:
        """One SweepResult over ``freqs`` from results on the index sets idx_a and idx_b."""
        nf, npo = len(freqs), len(self.ports)
        X = torch.empty((self.sys.n, nf, npo), dtype=torch.complex128, device=self.device)
        X[:, idx_a] = res_a.solutions.reshape(self.sys.n, len(idx_a), npo)
        X[:, idx_b] = res_b.solutions.reshape(self.sys.n, len(idx_b), npo)
        S = np.empty((nf, npo, npo), dtype=np.complex128)
        S[idx_a], S[idx_b] = res_a.S, res_b.S
        its = np.empty((nf, npo), dtype=np.int64)
        its[idx_a], its[idx_b] = res_a.iterations, res_b.iterations
        rs = np.empty((nf, npo))
        rs[idx_a], rs[idx_b] = res_a.residuals, res_b.residuals
        return SweepResult(freqs, S, its, rs, res_a.seconds + res_b.seconds, X.reshape(self.sys.n, nf * npo),
                           dict(res_b.info))

    def run_warm(self, freqs, n_train: int = 32, tol: float = 1e-10, restart: int = 150, max_iter: int = 20000,
                 chunk: int | None = None, guess: str = "projection", solver: str = "ilu0", n_anchor: int = 4,
                 precision: str = "fp32", mlp_steps: int = 1500, refine: int = 0, inner: str = "fp64",
                 mlp_target: str = "solutions") -> SweepResult:
        """Batched sweep: solve n_train evenly spread points, build an initial guess for
        every point from their span (``guess`` = "projection": minimal residual;
        "mlp": the warm-start network, trained on ``mlp_target`` (see mlp_guess);
        "none": zero), then finish all points with
        batched GMRES.  ``solver``: "ilu0" (batched ILU(0)-GMRES) or "anchored"
        (FGMRES preconditioned by slab factors at n_anchor anchors, see run_anchored)."""
        freqs = np.asarray(freqs, dtype=float)
        nf, npo = len(freqs), len(self.ports)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        tr = np.unique(np.round(np.linspace(0, nf - 1, min(n_train, nf))).astype(int))
        if solver == "anchored":
            anchors = self.default_anchors(freqs, n_anchor)
            solve = lambda fr, x0=None: self.run_anchored(fr, anchors=anchors, precision=precision, tol=tol,  # noqa: E731
                                                           restart=min(restart, 60), max_iter=max_iter, x0=x0,
                                                           chunk=chunk, refine=refine, inner=inner)
        else:
            solve = lambda fr, x0=None: self.run(fr, method="batched", tol=tol, restart=restart,  # noqa: E731
                                                 max_iter=max_iter, x0=x0, chunk=chunk)
        first = solve(freqs[tr])
        mlp_loss = None
        torch.cuda.synchronize()
        tg = time.perf_counter()
        if guess == "mlp":
            X0, mlp_loss = self.mlp_guess(first.solutions, freqs[tr], freqs, steps=mlp_steps, target=mlp_target)
        elif guess == "projection":
            X0 = self.project(first.solutions, freqs)
        else:
            X0 = None
        torch.cuda.synchronize()
        t_guess = time.perf_counter() - tg
        # the training points are done: solve the others and keep their solutions
        others = np.setdiff1d(np.arange(nf), tr)
        x0_others = None if X0 is None else X0.reshape(-1, nf, npo)[:, others].reshape(X0.shape[0], -1)
        if others.size:
            rest_part = solve(freqs[others], x0_others)
            rest = self._merge(freqs, tr, first, others, rest_part)
            final_s = rest_part.seconds
        else:                      # every point was a training point
            rest_part, rest, final_s = first, first, 0.0
        torch.cuda.synchronize()
        secs = time.perf_counter() - t0
        info = {"train_points": len(tr), "train_index": tr, "train_iterations": first.iterations,
                "train_seconds": first.seconds, "guess_seconds": t_guess, "final_seconds": final_s,
                "final_index": others, "final_iterations_mean": float(rest_part.iterations.mean()) if others.size else 0.0,
                "guess": guess, "mlp_loss": mlp_loss, "solver": solver,
                **({k: v for k, v in first.info.items()} if solver == "anchored" else {})}
        return SweepResult(freqs, rest.S, rest.iterations, rest.residuals, secs, rest.solutions, info)


class _UnitRobin:
    """A Robin BC with gamma = 1 and U_inc = E_mode (unit matrix / unit forcing)."""

    def __init__(self, bc):
        self.bc = bc
        self.tags = bc.tags
        self._include_stiff = bc._include_stiff
        self._include_force = getattr(bc, "_include_force", False)
        if hasattr(bc, "port_number"):
            self.port_number = bc.port_number
        if hasattr(bc, "cs"):
            self.cs = bc.cs

    def get_gamma(self, k0):
        return 1.0 + 0j

    def get_inv_basis(self):
        return self.bc.get_inv_basis()

    def get_Uinc(self, x, y, k0):
        return np.asarray(self.bc.port_mode_3d(x, y, k0), dtype=np.complex128)


def _is_lumped(bc) -> bool:
    """A port with a voltage line: this package's LumpedPort, or the reference's once
    define_lumped_port_integration_points has set its ``vintline``."""
    return bool(getattr(bc, "v_integration", False)) and (
        hasattr(bc, "integration_line") or getattr(bc, "vintline", None) is not None)


def _lumped_line(bc, mesh):
    """(midpoints (3, n), steps (3, n)) of a lumped port's voltage line."""
    if hasattr(bc, "integration_line"):
        return bc.integration_line(mesh)
    ln = bc.vintline
    return np.array(ln.cmid), np.array([ln.dxs, ln.dys, ln.dzs])


def _lumped_amp(bc) -> float:
    """|U_inc| / (2 k0) of a lumped port: V/h * 376.7303 / Zs (fem/bc.py:711-713)."""
    return float(bc.voltage) / float(bc.height) * (376.7303 / float(bc.surfZ))


def _zmode(bc, k0) -> float:
    z = getattr(bc, "Zmode", None)
    return complex(z(k0)) if callable(z) else 376.730313412


def _port_const(field, bc, er, ur) -> np.ndarray:
    """Per port triangle, the weight of the S-parameter mode integrals
    (fem/physics/edm/emfreq3d.py:767-778): TEM sqrt(tr er / tr ur), TE 3 / tr ur,
    TM 3 / tr er, with the material of the face's first tet (emfreq3d.py:480-486)."""
    m = field.mesh
    tri = np.asarray(m.get_triangles(bc.tags), dtype=np.int64)
    tet = np.asarray(m.tri_to_tet, dtype=np.int64)[0, tri]
    er = np.asarray(er)
    ur = np.asarray(ur)
    tre = er[0, 0, tet] + er[1, 1, tet] + er[2, 2, tet]
    tru = ur[0, 0, tet] + ur[1, 1, tet] + ur[2, 2, tet]
    kind = getattr(bc, "modetype", "TEM")
    if kind == "TE":
        return (1.0 / (tru / 3)).astype(np.complex128)
    if kind == "TM":
        return (1.0 / (tre / 3)).astype(np.complex128)
    return (1.0 / np.sqrt(tru / tre)).astype(np.complex128)


def _mode_power(field, bc, const=None) -> complex:
    """int const |E_mode|^2 over the port face with the 6-point rule (fem/mth/sparam.py:72-100)."""
    from .freq import dunavant6
    m = field.mesh
    tri = np.asarray(m.get_triangles(bc.tags), dtype=np.int64)
    tv = np.asarray(m.tris)[:, tri]
    nodes = np.asarray(m.nodes)
    D = dunavant6()
    v1, v2, v3 = nodes[:, tv[0]], nodes[:, tv[1]], nodes[:, tv[2]]
    area = np.linalg.norm(np.cross((v2 - v1).T, (v3 - v1).T), axis=1) / 2
    tot = 0.0
    for k in range(D.shape[1]):
        p = v1 * D[1, k] + v2 * D[2, k] + v3 * D[3, k]
        Em = bc.port_mode_3d_global(p[0], p[1], p[2], 1.0)
        w = area if const is None else area * const
        tot += D[0, k] * np.sum(np.sum(np.abs(Em) ** 2, axis=0) * w)
    return float(tot) if const is None else complex(tot)
