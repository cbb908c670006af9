"""Drop-ins for the reference's solve-routine and eigensolver slots.

``GPUSweepRoutine`` takes the place of ``physics.solveroutine`` (a ``SolveRoutine``,
fem/solver.py:361-469) under ``Electrodynamics3D.frequency_domain``
(fem/physics/edm/emfreq3d.py:607-732), which stays unmodified.  That driver assembles
K(k0) one frequency at a time and calls ``solve(K, b, solve_ids, reuse)`` once per
(frequency, active port), with ``reuse=False`` on the first port of every frequency
(emfreq3d.py:686-697).  Per call there is nothing to batch, so on its first call the
routine solves the whole sweep at once on the GPU (``FrequencySweep``: every
frequency x port column in one batched, mixed-precision, warm-started solve) and then
answers each call from that result.  Before it returns a column it checks it in FP64
against the matrix it was handed: ||K x - b|| / ||b|| over the solve DOFs must be at
most ``check_tol``.  A column that fails the check (a call sequence other than the
sweep's, a modified K) is solved on its own by ``GPUSolver`` from the handed matrix.

``GPUEigSolver`` fills the ``direct_eig_solver`` / ``iterative_eig_solver`` slots of a
``SolveRoutine`` (fem/solver.py:117-131, 471-505):

* ``iterative=False`` stands where ``SolverLAPACK.eig`` (fem/solver.py:310-341) does:
  dense A x = lambda B x, all eigenpairs, then the reference's ``filter_real_modes``
  (fem/solver.py:34-68) with its er_max = ur_max = 2.  The eigenvalues come from the
  shifted inverse (A - s B)^-1 B, s = -target_k0^2 (a GPU LU solve and the library's
  dense eigensolver on the device), lambda = s + 1/mu, which tolerates a singular B
  as QZ does.
* ``iterative=True`` stands where ``SolverARPACK.eig`` (fem/solver.py:343-357) does:
  the ``nmodes`` eigenvalues nearest sigma = -target_k0^2 (``eigsh(A, k, M=B, sigma,
  which)``) by shift-invert block Arnoldi on the slab factorization of A - sigma B
  (``ShiftInvertEigen``); real parts are returned, as eigsh returns them.
"""
from __future__ import annotations

import time

import numpy as np
import torch

from .solver import GPUSolver

C0 = 299792458.0


class GPUSweepRoutine:
    """``SolveRoutine`` drop-in that serves a frequency sweep from one batched GPU solve.

    Args:
        physics: the ``Electrodynamics3D`` object whose ``frequency_domain`` will call this
            routine; its ``basis``, ``boundary_conditions``, ``frequencies`` and materials
            (``mesh.retreive`` over ``mesher.volumes``, as emfreq3d.py:614-615) are read on
            the first call.  Or give ``field``, ``er``, ``ur``, ``bcs`` and ``frequencies``.
        method: "warm" (default: FP32 slab anchors, projection warm start), "anchored"
            (same without the warm start) or "plain" (one FP64 slab factorization per
            frequency).
        tol: FP64 relative residual every column is solved to.
        check_tol: FP64 relative residual a served column must meet against the handed K.
        sweep_kw: passed to ``FrequencySweep.run_warm`` / ``run_anchored``.
    """

    real_only = False

    def __init__(self, physics=None, *, field=None, er=None, ur=None, bcs=None, frequencies=None,
                 method: str = "warm", tol: float = 1e-10, check_tol: float = 1e-8, device="cuda", **sweep_kw):
        if method not in ("warm", "anchored", "plain"):
            raise ValueError(f"GPUSweepRoutine: unknown method {method!r}")
        self.physics = physics
        self._given = dict(field=field, er=er, ur=ur, bcs=bcs, frequencies=frequencies)
        self.method = method
        self.tol = tol
        self.check_tol = check_tol
        self.device = torch.device(device)
        self.sweep_kw = sweep_kw
        # the slots a SolveRoutine carries (fem/solver.py:361-381)
        self.direct_solver = GPUSolver(tol=tol, device=device)
        self.iterative_solver = self.direct_solver
        self.direct_eig_solver = GPUEigSolver(iterative=False, device=device)
        self.iterative_eig_solver = GPUEigSolver(iterative=True, device=device)
        self.use_sorter = False
        self.use_preconditioner = False
        self.use_direct = True
        self.reset()

    def __str__(self):
        return f"GPUSweepRoutine({self.method})"

    def reset(self):
        """Forget the cached sweep (the next call solves the sweep again)."""
        self._X = None
        self._f = -1
        self.sweep = None
        self.result = None
        self.stats = {"served": 0, "solved_alone": 0, "max_check_residual": 0.0, "sweep_seconds": 0.0}

    # ---------------------------------------------------------------- inputs ---
    def _inputs(self):
        g = dict(self._given)
        ph = self.physics
        if ph is not None:
            g["field"] = g["field"] if g["field"] is not None else ph.basis
            g["bcs"] = g["bcs"] if g["bcs"] is not None else ph.boundary_conditions
            g["frequencies"] = g["frequencies"] if g["frequencies"] is not None else ph.frequencies
            if g["er"] is None:
                g["er"] = ph.mesh.retreive(lambda mat, x, y, z: mat.fer3d_mat(x, y, z), ph.mesher.volumes)
            if g["ur"] is None:
                g["ur"] = ph.mesh.retreive(lambda mat, x, y, z: mat.fur3d_mat(x, y, z), ph.mesher.volumes)
        missing = [k for k, v in g.items() if v is None]
        if missing:
            raise ValueError(f"GPUSweepRoutine: missing {missing} (give physics= or the arrays)")
        return g

    def _run_sweep(self, solve_ids):
        from .freq import Assembler
        from .solver import FrequencySweep
        g = self._inputs()
        freqs = np.asarray(g["frequencies"], dtype=float)
        sw = FrequencySweep(Assembler(self.device), g["field"], g["er"], g["ur"], g["bcs"])
        if not np.array_equal(np.asarray(sw.solve_ids), np.asarray(solve_ids)):
            raise ValueError("GPUSweepRoutine: the handed solve_ids differ from the PEC set of the boundary "
                             "conditions")
        t0 = time.perf_counter()
        if self.method == "warm":
            kw = dict(n_train=12, solver="anchored", n_anchor=2, precision="fp32", guess="projection")
            kw.update(self.sweep_kw)
            res = sw.run_warm(freqs, tol=self.tol, **kw)
        elif self.method == "anchored":
            kw = dict(n_anchor=2, precision="fp32")
            kw.update(self.sweep_kw)
            res = sw.run_anchored(freqs, tol=self.tol, **kw)
        else:
            res = sw.run(freqs, method="plain", precond="slab64", tol=self.tol)
        self.stats["sweep_seconds"] = time.perf_counter() - t0
        self.sweep, self.result = sw, res
        self.freqs = freqs
        self._X = sw.sys.scatter(res.solutions)            # (nf * np, N) full DOF numbering, zeros on PEC
        # each port's forcing support, to tell which port drives a right-hand side
        self._support = [(sw.u[bc.port_number] != 0).cpu().numpy() for bc in sw.ports]

    # ----------------------------------------------------------------- solve ---
    def _port_of(self, b) -> int:
        nz = np.flatnonzero(b)
        hits = [i for i, m in enumerate(self._support) if nz.size and np.all(m[nz])]
        return hits[0] if len(hits) == 1 else -1

    def solve(self, A, b, solve_ids, reuse: bool = False) -> np.ndarray:
        """SolveRoutine.solve (fem/solver.py:405-469): the full-length solution, zeros on the
        DOFs outside ``solve_ids``."""
        from scipy.sparse import csr_matrix
        b = np.asarray(b, dtype=np.complex128)
        sid = np.asarray(solve_ids)
        if self._X is None:
            self._run_sweep(sid)
        if not reuse:
            self._f += 1
        npo = len(self.sweep.ports)
        p = self._port_of(b)
        K = csr_matrix(A)
        if 0 <= self._f < len(self.freqs) and p >= 0:
            x = self._X[self._f * npo + p].cpu().numpy()
            r = (K @ x)[sid] - b[sid]
            rel = float(np.linalg.norm(r) / max(np.linalg.norm(b[sid]), 1e-300))
            if rel <= self.check_tol:
                self.stats["served"] += 1
                self.stats["max_check_residual"] = max(self.stats["max_check_residual"], rel)
                return x
        # not a column of the sweep: solve the handed system on its own
        Asel = K[sid][:, sid]
        xs, info = self.direct_solver.solve(Asel, b[sid], None, reuse_factorization=False)
        if info < 0:
            raise RuntimeError(f"GPUSweepRoutine: solve failed (info {info})")
        out = np.zeros(A.shape[0], dtype=np.complex128)
        out[sid] = xs
        self.stats["solved_alone"] += 1
        return out

    def eig(self, A, B, solve_ids, nmodes: int = 6, direct: bool | None = None, target_k0: float | None = None,
            which: str = "LM"):
        """SolveRoutine.eig (fem/solver.py:471-505) with the GPU eigensolver slots."""
        sid = np.asarray(solve_ids)
        Asel = A.tocsr()[sid][:, sid] if hasattr(A, "tocsr") else np.asarray(A)[np.ix_(sid, sid)]
        Bsel = B.tocsr()[sid][:, sid] if hasattr(B, "tocsr") else np.asarray(B)[np.ix_(sid, sid)]
        solver = self.direct_eig_solver if (direct is None or direct) else self.iterative_eig_solver
        return solver.eig(Asel, Bsel, nmodes, target_k0, which)


def filter_real_modes(lam: np.ndarray, k0: float, ermax: float = 2.0, urmax: float = 2.0):
    """The reference's mode filter (fem/solver.py:34-68): -2 k0^2 er_max ur_max <= lambda <= -1,
    ordered by |sqrt(-lambda) - k0|; comparisons on the real part.  Returns (values, indices)."""
    lr = lam.real
    keep = np.flatnonzero((lr <= -1) & (lr >= -(k0 ** 2) * ermax * urmax * 2))
    order = np.argsort(np.abs(np.sqrt(-lam[keep]) - k0))
    keep = keep[order]
    return lam[keep], keep


class GPUEigSolver:
    """``Solver`` with ``eig(A, B, nmodes, target_k0, which)`` on the GPU (see the module text)."""

    real_only = False
    req_sorter = False

    def __init__(self, iterative: bool = False, device="cuda", tol: float = 1e-10):
        self.own_preconditioner = True
        self.iterative = iterative
        self.device = torch.device(device)
        self.tol = tol
        self.last_info = {}

    def __str__(self):
        return "GPUEigSolver(iterative)" if self.iterative else "GPUEigSolver(direct)"

    def solve(self, A, b, precon=None, reuse_factorization: bool = False):
        return GPUSolver(tol=self.tol, device=self.device).solve(A, b, precon, reuse_factorization)

    def eig(self, A, B, nmodes: int = 6, target_k0: float | None = 0.0, which: str = "LM"):
        k0 = float(target_k0 or 0.0)
        if self.iterative:
            return self._eig_sparse(A, B, nmodes, k0, which)
        return self._eig_dense(A, B, k0)

    def _eig_dense(self, A, B, k0: float):
        dev = self.device
        Ad = torch.as_tensor(A.toarray() if hasattr(A, "toarray") else np.asarray(A), dtype=torch.complex128,
                             device=dev)
        Bd = torch.as_tensor(B.toarray() if hasattr(B, "toarray") else np.asarray(B), dtype=torch.complex128,
                             device=dev)
        sigma = -k0 * k0 if k0 != 0.0 else -1.0
        mu, vec = torch.linalg.eig(torch.linalg.solve(Ad - sigma * Bd, Bd))
        mu = mu.cpu().numpy()
        lam = np.full(mu.shape, np.inf + 0j)
        finite = np.abs(mu) > 1e-12 * max(np.abs(mu).max(), 1e-300)
        lam[finite] = sigma + 1.0 / mu[finite]
        vals, keep = filter_real_modes(lam, k0)
        self.last_info = {"n": int(Ad.shape[0]), "sigma": sigma, "found": int(keep.size)}
        return vals, vec[:, torch.as_tensor(keep, device=dev)].cpu().numpy()

    def _eig_sparse(self, A, B, nmodes: int, k0: float, which: str):
        from scipy.sparse import csr_matrix
        from .eigen import ShiftInvertEigen
        from .solver import RestrictedSystem, SlabFactor
        dev = self.device
        A = csr_matrix(A)
        B = csr_matrix(B)
        n = A.shape[0]
        P = (abs(A) + abs(B)).tocsr()
        P.sort_indices()
        rows = np.repeat(np.arange(n), np.diff(P.indptr))
        av = np.asarray(A[rows, P.indices]).ravel().astype(np.complex128)
        bv = np.asarray(B[rows, P.indices]).ravel().astype(np.complex128)
        sysr = RestrictedSystem(torch.as_tensor(P.indptr.astype(np.int64), device=dev),
                                torch.as_tensor(P.indices.astype(np.int32), device=dev), P.nnz, np.arange(n))
        a = torch.as_tensor(av, device=dev)
        bb = torch.as_tensor(bv, device=dev)
        z = torch.zeros_like(a)
        Er = sysr.form(a, z, [0.0])
        Br = sysr.form(z, bb, [-1.0])
        sigma = -k0 * k0
        eig = ShiftInvertEigen(sysr, Er, Br, SlabFactor(sysr))
        r = eig.solve(nmodes, sigma, which=which)
        self.last_info = {"n": n, "sigma": sigma, "residuals": r.residuals, **r.info}
        return r.eigenvalues.real, r.vectors.cpu().numpy()
