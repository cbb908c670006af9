"""GPU drop-in for EMerge's tetrahedral assembler.

``tet_mass_stiffness_matrices(field, er, ur)`` has the signature and return
value of fem/physics/edm/optimized_assembly.py:43-64: it integrates the
second-order Nédélec curl-curl matrix E (weighted by μr⁻¹) and mass matrix B
(weighted by εr) of every tetrahedron and returns both as SciPy CSR matrices
with the pattern of ``coo_matrix(...).tocsr()`` (sorted indices, duplicates
summed, explicit zeros kept).  The integration and the summation run on the GPU
through the C ABI (``emg_plan_create`` / ``emg_assemble_tet``).

Install into an EMerge session (the assembler looks the function up lazily,
fem/physics/edm/assembler.py:319)::

    import fem.physics.edm.optimized_assembly as oa
    from emerge_gb300.assembly import tet_mass_stiffness_matrices
    oa.tet_mass_stiffness_matrices = tet_mass_stiffness_matrices

Materials: when εr and μr are scalar multiples of the identity in every tet the
float-float fill runs (``emg_assemble_tet``); any other (3,3,nT) tensors go to
the FP64 tensor fill (``emg_assemble_tet_tensor``) with Ms = matinv(μr) and
Mm = εr per tet, as _matrix_builder passes them (optimized_assembly.py:95-108).
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib


def _dptr(t: torch.Tensor) -> ctypes.c_void_p:
    return ctypes.c_void_p(t.data_ptr())


def _stream() -> ctypes.c_void_p:
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _check_tensor(m: np.ndarray, name: str) -> np.ndarray:
    m = np.asarray(m)
    if m.ndim != 3 or m.shape[:2] != (3, 3):
        raise ValueError(f"{name} must have shape (3, 3, n_tets), got {m.shape}")
    return m


def is_scalar_material(m: np.ndarray) -> bool:
    """True when every tet's (3,3) tensor is s·I."""
    m = np.asarray(m)
    d = m[0, 0, :]
    off = np.abs(m[0, 1]) + np.abs(m[0, 2]) + np.abs(m[1, 0]) + np.abs(m[1, 2]) + np.abs(m[2, 0]) + np.abs(m[2, 1])
    return not (np.any(off != 0) or np.any(m[1, 1] != d) or np.any(m[2, 2] != d))


def scalar_material(m: np.ndarray, name: str) -> np.ndarray:
    """Return the per-tet scalar of a (3,3,nT) material tensor that is s·I, else raise."""
    m = _check_tensor(m, name)
    if not is_scalar_material(m):
        raise ValueError(f"{name} is not a scalar multiple of the identity in every tet")
    return m[0, 0, :].astype(np.complex128)


def matinv_device(s: torch.Tensor) -> torch.Tensor:
    """matinv (fem/mth/optimized.py:440-461) on the GPU (``emg_matinv``): ``s`` complex128
    CUDA tensor (9, n_tets) (the reference's (3,3,n) in C order) or (n_tets,) scalars
    (isotropic tensors s*I, whose matinv is 1/s)."""
    s = s.contiguous()
    assert s.dtype == torch.complex128 and s.is_cuda
    ncomp = 9 if s.dim() == 2 else 1
    n = int(s.shape[-1])
    out = torch.empty_like(s)
    with torch.cuda.device(s.device):
        _lib.call("emg_matinv", n, ncomp, _dptr(s), _dptr(out), _stream())
    return out


def matinv_tensors(s: np.ndarray) -> np.ndarray:
    """matinv (fem/mth/optimized.py:441-461) of every (3,3) slice of a (3,3,nT) array.

    A tensor with all off-diagonal entries zero gets the reciprocal diagonal;
    any other gets adj(s)·det(s), the reference's expression (it multiplies by
    the determinant rather than dividing).
    """
    s = np.asarray(s, dtype=np.complex128)
    out = np.zeros_like(s)
    diag = ((s[0, 1] == 0) & (s[0, 2] == 0) & (s[1, 0] == 0) & (s[1, 2] == 0) & (s[2, 0] == 0) & (s[2, 1] == 0))
    with np.errstate(divide="ignore", invalid="ignore"):
        for k in range(3):
            out[k, k] = np.where(diag, 1 / s[k, k], 0)
    g = ~diag
    if np.any(g):
        a = s[:, :, g]
        det = (a[0, 0] * a[1, 1] * a[2, 2] - a[0, 0] * a[1, 2] * a[2, 1] - a[0, 1] * a[1, 0] * a[2, 2]
               + a[0, 1] * a[1, 2] * a[2, 0] + a[0, 2] * a[1, 0] * a[2, 1] - a[0, 2] * a[1, 1] * a[2, 0])
        adj = np.empty_like(a)
        adj[0, 0] = a[1, 1] * a[2, 2] - a[1, 2] * a[2, 1]
        adj[0, 1] = -a[0, 1] * a[2, 2] + a[0, 2] * a[2, 1]
        adj[0, 2] = a[0, 1] * a[1, 2] - a[0, 2] * a[1, 1]
        adj[1, 0] = -a[1, 0] * a[2, 2] + a[1, 2] * a[2, 0]
        adj[1, 1] = a[0, 0] * a[2, 2] - a[0, 2] * a[2, 0]
        adj[1, 2] = -a[0, 0] * a[1, 2] + a[0, 2] * a[1, 0]
        adj[2, 0] = a[1, 0] * a[2, 1] - a[1, 1] * a[2, 0]
        adj[2, 1] = -a[0, 0] * a[2, 1] + a[0, 1] * a[2, 0]
        adj[2, 2] = a[0, 0] * a[1, 1] - a[0, 1] * a[1, 0]
        out[:, :, g] = adj * det
    return out


class AssemblyPlan:
    """Device-resident assembly plan of one mesh (CSR pattern + tet geometry).

    Args:
        field: a Nedelec2-like object (``field.mesh`` with nodes, tets, tris,
            edges, edge_lengths, tet_to_edge; ``field.tet_to_field``).
        device: CUDA device.
    """

    def __init__(self, field, device: str | torch.device = "cuda"):
        lib = _lib.load()
        m = field.mesh
        self.device = torch.device(device)
        dev = self.device

        def i32(a):
            return torch.as_tensor(np.ascontiguousarray(a, dtype=np.int32), device=dev)

        def f64(a):
            return torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64), device=dev)

        # the arrays this plan was built from: a field whose mesh arrays were
        # replaced (moved nodes, a new mesh of the same size) gets a new plan
        self._source = (m.nodes, m.tets, m.edges, m.tris, field.tet_to_field)
        self.n_tets = int(m.tets.shape[1])
        self.n_edges = int(m.edges.shape[1])
        self.n_tris = int(m.tris.shape[1])
        self.n_field = 2 * self.n_edges + 2 * self.n_tris
        nodes = f64(m.nodes)
        tets = i32(m.tets)
        edges = i32(m.edges)
        tris = i32(m.tris)
        t2f = i32(field.tet_to_field)
        t2e = i32(m.tet_to_edge)
        el = f64(m.edge_lengths)
        plan = ctypes.c_void_p()
        with torch.cuda.device(dev):
            _lib.call("emg_plan_create", self.n_nodes_of(m), self.n_tets, self.n_edges, self.n_tris, self.n_field,
                      _dptr(nodes), _dptr(tets), _dptr(edges), _dptr(tris), _dptr(t2f), _dptr(t2e), _dptr(el),
                      _stream(), ctypes.byref(plan))
        self._plan = plan
        self._lib = lib
        self.nnz = int(lib.emg_plan_nnz(plan))
        self.indptr = torch.empty(self.n_field + 1, dtype=torch.int64, device=dev)
        self.indices = torch.empty(max(self.nnz, 1), dtype=torch.int32, device=dev)
        with torch.cuda.device(dev):
            _lib.call("emg_plan_pattern", plan, _dptr(self.indptr), _dptr(self.indices), _stream())
        self._host_pattern = None

    def matches(self, field) -> bool:
        """True when ``field`` still holds the very arrays this plan was built from."""
        m = field.mesh
        now = (m.nodes, m.tets, m.edges, m.tris, field.tet_to_field)
        return all(a is b for a, b in zip(self._source, now))

    @staticmethod
    def n_nodes_of(m) -> int:
        return int(m.nodes.shape[1])

    def __del__(self):
        p = getattr(self, "_plan", None)
        if p is not None and p.value:
            try:
                self._lib.emg_plan_destroy(p)
            except Exception:
                pass
            self._plan = None

    def pattern_host(self):
        if self._host_pattern is None:
            ip = self.indptr.cpu().numpy()
            ix = self.indices[: self.nnz].cpu().numpy()
            idx_t = np.int32 if self.nnz < 2 ** 31 and self.n_field < 2 ** 31 else np.int64
            self._host_pattern = (ip.astype(idx_t), ix.astype(idx_t))
        return self._host_pattern

    def rows_host(self, rows, *values: torch.Tensor):
        """Rows ``rows`` of device CSR value arrays on this plan's pattern, copied to the host:
        (indptr, indices, *values) of the (len(rows), N) row block."""
        r = torch.as_tensor(np.asarray(rows, dtype=np.int64), device=self.device)
        start, stop = self.indptr[r], self.indptr[r + 1]
        cnt = stop - start
        ip = torch.zeros(len(r) + 1, dtype=torch.int64, device=self.device)
        ip[1:] = torch.cumsum(cnt, 0)
        owner = torch.repeat_interleave(torch.arange(len(r), device=self.device), cnt)
        pos = start[owner] + (torch.arange(int(ip[-1]), device=self.device) - ip[:-1][owner])
        return (ip.cpu().numpy(), self.indices[pos].cpu().numpy(), *(v[pos].cpu().numpy() for v in values))

    def assemble(self, eps: torch.Tensor, mu_inv: torch.Tensor, E: torch.Tensor | None = None,
                 B: torch.Tensor | None = None):
        """Device call: eps, mu_inv complex128 (n_tets,) CUDA tensors -> (E, B) complex128 (nnz,)."""
        if E is None:
            E = torch.empty(max(self.nnz, 1), dtype=torch.complex128, device=self.device)
        if B is None:
            B = torch.empty(max(self.nnz, 1), dtype=torch.complex128, device=self.device)
        assert eps.dtype == torch.complex128 and mu_inv.dtype == torch.complex128
        assert eps.is_contiguous() and mu_inv.is_contiguous() and E.is_contiguous() and B.is_contiguous()
        with torch.cuda.device(self.device):
            _lib.call("emg_assemble_tet", self._plan, _dptr(eps), _dptr(mu_inv), _dptr(E), _dptr(B), _stream())
        return E, B

    def assemble_tensor(self, eps9: torch.Tensor, mu_inv9: torch.Tensor, E: torch.Tensor | None = None,
                        B: torch.Tensor | None = None):
        """Device call for tensor materials: eps9, mu_inv9 complex128 (9, n_tets) CUDA tensors."""
        if E is None:
            E = torch.empty(max(self.nnz, 1), dtype=torch.complex128, device=self.device)
        if B is None:
            B = torch.empty(max(self.nnz, 1), dtype=torch.complex128, device=self.device)
        for t in (eps9, mu_inv9):
            assert t.dtype == torch.complex128 and t.is_contiguous() and tuple(t.shape) == (9, self.n_tets)
        with torch.cuda.device(self.device):
            _lib.call("emg_assemble_tet_tensor", self._plan, _dptr(eps9), _dptr(mu_inv9), _dptr(E), _dptr(B),
                      _stream())
        return E, B

    def assemble_tensor_host(self, eps9: np.ndarray, mu_inv9: np.ndarray):
        """Host call through emg_assemble_tet_tensor_host: (9, n_tets) complex numpy in, values out."""
        eps9 = np.ascontiguousarray(eps9, dtype=np.complex128).reshape(9, self.n_tets)
        mu_inv9 = np.ascontiguousarray(mu_inv9, dtype=np.complex128).reshape(9, self.n_tets)
        E = np.empty(self.nnz, dtype=np.complex128)
        B = np.empty(self.nnz, dtype=np.complex128)
        with torch.cuda.device(self.device):
            _lib.call("emg_assemble_tet_tensor_host", self._plan, eps9.ctypes.data_as(ctypes.c_void_p),
                      mu_inv9.ctypes.data_as(ctypes.c_void_p), E.ctypes.data_as(ctypes.c_void_p),
                      B.ctypes.data_as(ctypes.c_void_p), _stream())
        return E, B

    def assemble_materials(self, er: np.ndarray, ur: np.ndarray):
        """Device values (E, B) for (3,3,nT) host material arrays; scalar or tensor fill as they require."""
        er = _check_tensor(er, "er")
        ur = _check_tensor(ur, "ur")
        if is_scalar_material(er) and is_scalar_material(ur):
            eps = scalar_material(er, "er")
            mu = scalar_material(ur, "ur")
            return self.assemble(torch.as_tensor(eps, device=self.device),
                                 matinv_device(torch.as_tensor(mu, device=self.device)))
        eps9 = np.ascontiguousarray(er, dtype=np.complex128).reshape(9, -1)
        ur9 = np.ascontiguousarray(ur, dtype=np.complex128).reshape(9, -1)
        return self.assemble_tensor(torch.as_tensor(eps9, device=self.device),
                                    matinv_device(torch.as_tensor(ur9, device=self.device)))

    def assemble_host(self, eps: np.ndarray, mu_inv: np.ndarray, E: np.ndarray | None = None,
                      B: np.ndarray | None = None):
        """Host call through emg_assemble_tet_host: numpy in, numpy out (copies inside the call)."""
        eps = np.ascontiguousarray(eps, dtype=np.complex128)
        mu_inv = np.ascontiguousarray(mu_inv, dtype=np.complex128)
        if E is None:
            E = np.empty(self.nnz, dtype=np.complex128)
        if B is None:
            B = np.empty(self.nnz, dtype=np.complex128)
        with torch.cuda.device(self.device):
            _lib.call("emg_assemble_tet_host", self._plan, eps.ctypes.data_as(ctypes.c_void_p),
                      mu_inv.ctypes.data_as(ctypes.c_void_p), E.ctypes.data_as(ctypes.c_void_p),
                      B.ctypes.data_as(ctypes.c_void_p), _stream())
        return E, B


def plan_for(field, device: str | torch.device = "cuda") -> AssemblyPlan:
    """The cached plan of ``field`` (built on first use)."""
    plan = getattr(field, "_emg_assembly_plan", None)
    if plan is None or not plan.matches(field):
        plan = AssemblyPlan(field, device)
        try:
            field._emg_assembly_plan = plan
        except AttributeError:
            pass
    return plan


def material_scalars(er: np.ndarray, ur: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """(eps, mu_inv) per tet: er = eps·I and matinv(ur) = (1/ur)·I (fem/mth/optimized.py:444-447)."""
    eps = scalar_material(er, "er")
    mu = scalar_material(ur, "ur")
    return eps, 1.0 / mu


def tet_mass_stiffness_matrices(field, er: np.ndarray, ur: np.ndarray):
    """Drop-in for fem/physics/edm/optimized_assembly.py:43-64 -> (E, B) scipy CSR, complex128."""
    from scipy.sparse import csr_matrix
    plan = plan_for(field)
    er = _check_tensor(er, "er")
    ur = _check_tensor(ur, "ur")
    if is_scalar_material(er) and is_scalar_material(ur):
        eps = scalar_material(er, "er")
        mu = torch.as_tensor(scalar_material(ur, "ur"), device=plan.device)
        mu_inv = matinv_device(mu).cpu().numpy()
        Ed, Bd = plan.assemble_host(eps, mu_inv)
    else:
        ur9 = torch.as_tensor(np.ascontiguousarray(ur, dtype=np.complex128).reshape(9, -1), device=plan.device)
        Ed, Bd = plan.assemble_tensor_host(np.ascontiguousarray(er, dtype=np.complex128).reshape(9, -1),
                                           matinv_device(ur9).cpu().numpy())
    ip, ix = plan.pattern_host()
    N = plan.n_field
    E = csr_matrix((Ed, ix, ip), shape=(N, N))
    B = csr_matrix((Bd, ix.copy(), ip.copy()), shape=(N, N))
    E.has_sorted_indices = True
    B.has_sorted_indices = True
    return E, B
