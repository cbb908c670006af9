"""GPU frequency-matrix assembly: drop-in for the reference Assembler.

``Assembler.assemble_freq_matrix(field, er, ur, bcs, frequency, cache_matrices)``
keeps the signature and outputs of fem/physics/edm/assembler.py:312-388:

* ``K = E - k0² B + Σ γ_p(k0) B_p`` (host SciPy CSR; the volume pattern with
  explicit zeros kept, where SciPy's ``+``/``-`` would drop exact zeros),
* ``b`` (zeros), ``solve_ids`` (DOFs not on PEC faces), ``port_vectors``.

E and B come from the GPU assembler (cached per mesh), the Robin blocks of
every port / absorbing triangle from ``emg_tri_robin_force`` /
``emg_tri_robin_abc``, and their summation into K and into the port vectors
from ``emg_segment_add`` with plan-time sorted segments (deterministic).  The
device-resident pieces (``DeviceSystem``) feed the GPU solver without a host
round trip.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib
from .assembly import AssemblyPlan, plan_for
from .bc import C0, is_pec, is_robin

# Dunavant order-4 rule (6 points) as weights and barycentrics, the rule
# gaus_quad_tri(4) expands to (fem/mth/optimized.py:28-29, 77-108).
_W1, _A1, _B1 = 0.223381589678011, 0.108103018168070, 0.445948490915965
_W2, _A2, _B2 = 0.109951743655322, 0.816847572980459, 0.091576213509771


def dunavant6() -> np.ndarray:
    """(4, 6): weights and barycentrics in the reference's point order."""
    pts = []
    for W, l1, l2, l3 in ((_W1, _A1, _B1, _B1), (_W2, _A2, _B2, _B2)):
        a, b, c = l1, l2, l3
        for _ in range(3):
            pts.append([W, a, b, c])
            a, b, c = b, c, a
    return np.array(pts).T


def _vp(t: torch.Tensor) -> ctypes.c_void_p:
    return ctypes.c_void_p(t.data_ptr())


def _stream() -> ctypes.c_void_p:
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


@dataclass
class _Segments:
    seg: torch.Tensor     # int64 (n_seg + 1)
    perm: torch.Tensor    # int64
    dst: torch.Tensor     # int64 (n_seg)

    @property
    def n(self) -> int:
        return int(self.dst.numel())


def _segments(keys: np.ndarray, device) -> _Segments:
    """Group ``keys`` (one per contribution, contribution index = position in the array)
    into segments of equal key, contributions in ascending index order."""
    order = np.argsort(keys, kind="stable")
    k = keys[order]
    starts = np.flatnonzero(np.r_[True, k[1:] != k[:-1]]) if len(k) else np.zeros(0, dtype=np.int64)
    seg = np.r_[starts, len(k)].astype(np.int64)
    return _Segments(torch.as_tensor(seg, device=device), torch.as_tensor(order.astype(np.int64), device=device),
                     torch.as_tensor(k[starts].astype(np.int64), device=device))


class _RobinPlan:
    """Per boundary condition: its triangles and the K / port-vector segment lists."""

    def __init__(self, field, plan: AssemblyPlan, tri_ids: np.ndarray):
        dev = plan.device
        m = field.mesh
        self.tri_ids = np.asarray(tri_ids, dtype=np.int64)
        self.n = len(self.tri_ids)
        t2f = np.asarray(field.tri_to_field, dtype=np.int64)[:, self.tri_ids]          # (8, n)
        rows = np.repeat(t2f.T, 8, axis=1).ravel()                                     # tri-major, row-major 8x8
        cols = np.tile(t2f.T, (1, 8)).ravel()
        r = torch.as_tensor(rows.astype(np.int32), device=dev)
        c = torch.as_tensor(cols.astype(np.int32), device=dev)
        pos = torch.empty(max(len(rows), 1), dtype=torch.int64, device=dev)
        with torch.cuda.device(dev):
            _lib.call("emg_csr_positions", len(rows), _vp(r), _vp(c), _vp(plan.indptr), _vp(plan.indices), _vp(pos),
                      _stream())
        p = pos[: len(rows)].cpu().numpy()
        if np.any(p < 0):
            raise ValueError("a boundary triangle's DOF pair is outside the volume CSR pattern")
        self.kseg = _segments(p, dev)
        self.vseg = _segments(t2f.T.ravel(), dev)                                      # forcing: tri-major 8
        self.tri_vertices = np.asarray(m.tris, dtype=np.int64)[:, self.tri_ids]


@dataclass
class DeviceSystem:
    """K(k0) on the volume CSR pattern plus port right-hand sides, resident on the GPU."""
    K: torch.Tensor                       # complex128 (nnz)
    indptr: torch.Tensor                  # int64 (N+1)
    indices: torch.Tensor                 # int32 (nnz)
    port_vectors: dict                    # port number -> complex128 (N)
    solve_ids: np.ndarray
    k0: float


class Assembler:
    """GPU drop-in for fem/physics/edm/assembler.py ``Assembler`` (frequency matrices)."""

    def __init__(self, device: str | torch.device = "cuda"):
        self.cached_matrices = None
        self.device = torch.device(device)
        # caches hold the field (and material arrays) they were built for, so an id is
        # never reused by another object while its entry lives
        self._dev = None           # (field, er, ur, plan, E, B)
        self._robin = {}           # (field id, tags) -> (field, _RobinPlan)
        self._solve_ids = {}       # (field id, pec tags) -> (field, solve_ids)
        self._dpts = dunavant6()
        self._dpts_dev = None

    # ---------------------------------------------------------------- volume ---
    def _volume(self, field, er, ur):
        """Device E and B of ``field`` for these material arrays (assembled again when
        either the field or a material array is a different object)."""
        d = self._dev
        if d is None or d[0] is not field or d[1] is not er or d[2] is not ur:
            plan = plan_for(field, self.device)
            E, B = plan.assemble_materials(er, ur)
            self._dev = (field, er, ur, plan, E, B)
        return self._dev[3], self._dev[4], self._dev[5]

    def _robin_plan(self, field, plan, bc):
        key = (id(field), tuple(bc.tags))
        hit = self._robin.get(key)
        if hit is None or hit[0] is not field:
            hit = (field, _RobinPlan(field, plan, field.mesh.get_triangles(bc.tags)))
            self._robin[key] = hit
        return hit[1]

    def solve_ids(self, field, bcs) -> np.ndarray:
        """DOFs not on PEC faces: 2 per PEC-face edge, 2 per PEC face (assembler.py:348-359, 384-385)."""
        pecs = [bc for bc in bcs if is_pec(bc)]
        key = (id(field), tuple(t for bc in pecs for t in bc.tags))
        hit = self._solve_ids.get(key)
        if hit is None or hit[0] is not field:
            m = field.mesh
            N = field.n_field
            mask = np.ones(N, dtype=bool)
            for pec in pecs:
                tri_ids = np.asarray(m.get_triangles(pec.tags), dtype=np.int64)
                if len(tri_ids) == 0:
                    continue
                edge_ids = np.asarray(m.tri_to_edge, dtype=np.int64)[:, tri_ids].ravel()
                mask[np.asarray(field.edge_to_field, dtype=np.int64)[:, edge_ids].ravel()] = False
                mask[np.asarray(field.tri_to_field, dtype=np.int64)[:, tri_ids].ravel()] = False
            hit = (field, np.flatnonzero(mask).astype(np.int64))
            self._solve_ids[key] = hit
        return hit[1]

    # ---------------------------------------------------------- per frequency ---
    def device_system(self, field, er, ur, bcs, frequency: float, force_weights: dict | None = None) -> DeviceSystem:
        """K(k0), port vectors and solve_ids on the device.  ``force_weights`` maps a port
        number to one complex weight per port triangle that scales its U_inc (used for the
        material-weighted S-parameter functionals of the sweep)."""
        plan, E, B = self._volume(field, er, ur)
        dev = self.device
        k0 = 2 * np.pi * frequency / C0
        N = plan.n_field
        K = torch.empty_like(E)
        with torch.cuda.device(dev):
            _lib.call("emg_combine", plan.nnz, _vp(E), _vp(B), ctypes.c_double(k0 ** 2), _vp(K), _stream())
        if self._dpts_dev is None:
            self._dpts_dev = torch.as_tensor(np.ascontiguousarray(self._dpts), device=dev)
        port_vectors = {}
        for bc in bcs:
            if hasattr(bc, "port_number") and hasattr(bc, "_include_force"):
                port_vectors[bc.port_number] = torch.zeros(N, dtype=torch.complex128, device=dev)
        m = field.mesh
        for bc in bcs:
            if not is_robin(bc):
                continue
            rp = self._robin_plan(field, plan, bc)
            if rp.n == 0:
                continue
            g = complex(bc.get_gamma(k0))
            Bblk = torch.empty(rp.n * 64, dtype=torch.complex128, device=dev)
            if bc._include_force:
                basis = bc.get_inv_basis()
                origin = np.asarray(bc.cs.origin, dtype=float)
                # vertices_local = local_basis @ (nodes - origin) (assembler.py:111)
                vloc = basis @ (np.asarray(m.nodes) - origin[:, None])
                lcs = np.ascontiguousarray(vloc[:2][:, rp.tri_vertices])                # (2, 3, n)
                D = self._dpts
                x = (lcs[0][:, None, :] * D[1:, :, None]).sum(axis=0)                   # (npts, n)
                y = (lcs[1][:, None, :] * D[1:, :, None]).sum(axis=0)
                # generate_points order: (npts, n) flattened (assembler.py:63-81)
                U = np.asarray(bc.get_Uinc(x.ravel(), y.ravel(), k0), dtype=np.complex128).reshape(3, D.shape[1], rp.n)
                if force_weights and bc.port_number in force_weights:
                    U = U * np.asarray(force_weights[bc.port_number], dtype=np.complex128)[None, None, :]
                lcs_d = torch.as_tensor(lcs, device=dev)
                U_d = torch.as_tensor(np.ascontiguousarray(U), device=dev)
                bblk = torch.empty(rp.n * 8, dtype=torch.complex128, device=dev)
                with torch.cuda.device(dev):
                    _lib.call("emg_tri_robin_force", rp.n, _vp(lcs_d), _vp(U_d), _vp(self._dpts_dev), D.shape[1],
                              ctypes.c_double(g.real), ctypes.c_double(g.imag), _vp(Bblk), _vp(bblk), _stream())
                    pv = port_vectors[bc.port_number]
                    s = rp.vseg
                    _lib.call("emg_segment_add", s.n, _vp(s.seg), _vp(s.perm), _vp(s.dst), _vp(bblk),
                              ctypes.c_double(1.0), ctypes.c_double(0.0), _vp(pv), _stream())
            else:
                tv = rp.tri_vertices
                xyz = np.ascontiguousarray(np.asarray(m.nodes)[:, tv])                 # (3, 3, n)
                el = np.ascontiguousarray(np.asarray(m.edge_lengths)[np.asarray(m.tri_to_edge)[:, rp.tri_ids]])
                xyz_d = torch.as_tensor(xyz, device=dev)
                el_d = torch.as_tensor(el, device=dev)
                with torch.cuda.device(dev):
                    _lib.call("emg_tri_robin_abc", rp.n, _vp(xyz_d), _vp(el_d), ctypes.c_double(g.real),
                              ctypes.c_double(g.imag), _vp(Bblk), _stream())
            if bc._include_stiff:
                s = rp.kseg
                with torch.cuda.device(dev):
                    _lib.call("emg_segment_add", s.n, _vp(s.seg), _vp(s.perm), _vp(s.dst), _vp(Bblk),
                              ctypes.c_double(1.0), ctypes.c_double(0.0), _vp(K), _stream())
        return DeviceSystem(K, plan.indptr, plan.indices[: plan.nnz], port_vectors, self.solve_ids(field, bcs), k0)

    def assemble_freq_matrix(self, field, er, ur, bcs, frequency, cache_matrices=False):
        """Drop-in for fem/physics/edm/assembler.py:312-388 -> (K, b, solve_ids, port_vectors) on the host."""
        from scipy.sparse import csr_matrix
        sysd = self.device_system(field, er, ur, bcs, frequency)
        plan = self._dev[3]
        ip, ix = plan.pattern_host()
        N = plan.n_field
        K = csr_matrix((sysd.K.cpu().numpy(), ix, ip), shape=(N, N))
        if cache_matrices and self.cached_matrices is None:
            E, B = self._dev[4], self._dev[5]
            self.cached_matrices = (csr_matrix((E.cpu().numpy(), ix, ip), shape=(N, N)),
                                    csr_matrix((B.cpu().numpy(), ix, ip), shape=(N, N)))
        b = np.zeros(N, dtype=np.complex128)
        pvs = {k: v.cpu().numpy() for k, v in sysd.port_vectors.items()}
        return K, b, sysd.solve_ids, pvs
