"""Waveguide-port modal analysis on the GPU (the reference's ModalPort mode solve).

``port_modes`` follows ``Electrodynamics3D.modal_analysis`` (fem/physics/edm/emfreq3d.py:201-365)
and ``Assembler.assemble_bma_matrices`` (fem/physics/edm/assembler.py:244-303):

1. The port face's triangles form a surface mesh (``Mesh3D.boundary_surface`` /
   ``SurfaceMesh``, fem/mesh3d.py:450-540): its nodes in ascending original order,
   edges (v0,v1), (v1,v2), (v0,v2) of each triangle.
2. The Nedelec-Lagrange-2 DOF map (fem/elements/nedleg2.py:32-70):
   [edge m1 | face m1 | edge m2 | face m2 | vertices | edge z], n_xy = 2 nE + 2 nT.
3. Element matrices on the GPU (``emg_port_element_matrices``), on the face's
   coordinates in the port frame (pinv(basis) @ nodes, nedeleclegrange2.py:41),
   with the materials of each face triangle's first tet; summed into dense A and B
   by a sorted (deterministic) coalesce.
4. PEC: every DOF of a face edge that lies on a PEC triangle (its two transverse
   DOFs, its z DOF and its two vertex DOFs, assembler.py:268-293) is removed.
5. A x = lambda B x on the remaining DOFs, dense: the reference calls LAPACK's
   generalized eig (fem/solver.py:316-341).  Here the shifted inverse
   (A - s B)^-1 B, s = -t^2, is formed by a GPU LU solve and its eigenvalues mu by
   the library's dense eigensolver on the device; lambda = s + 1/mu.  Like QZ this
   tolerates a singular B (its infinite eigenvalues become mu = 0).
6. Modes with -8 t^2 <= lambda <= -1 are kept and ordered by |sqrt(-lambda) - t|,
   t = the target propagation constant (filter_real_modes, fem/solver.py:34-68).

Returns the propagation constants beta = sqrt(-lambda) and the modes (full DOF
numbering, zeros on PEC DOFs).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib


def _vp(t: torch.Tensor) -> ctypes.c_void_p:
    return ctypes.c_void_p(t.data_ptr())


@dataclass
class PortSurface:
    """The surface mesh of a port face and its Nedelec-Lagrange-2 DOF map."""
    node_ids: np.ndarray        # (nN,) original node index of each surface node
    tris: np.ndarray            # (3, nT) surface node indices
    edges: np.ndarray           # (2, nE) surface node indices, ascending
    tri_to_edge: np.ndarray     # (3, nT): edges (v0,v1), (v1,v2), (v0,v2)
    tri_to_field: np.ndarray    # (14, nT)
    edge_to_field: np.ndarray   # (5, nE)
    n_field: int
    n_xy: int


def port_surface(mesh, tri_ids) -> PortSurface:
    tris3 = np.asarray(mesh.tris)[:, np.asarray(tri_ids, dtype=np.int64)]
    node_ids = np.unique(tris3.ravel())
    local = np.searchsorted(node_ids, tris3)
    nT = local.shape[1]
    nN = node_ids.size
    pairs = np.concatenate([local[[0, 1]], local[[1, 2]], local[[0, 2]]], axis=1)
    lo, hi = np.minimum(pairs[0], pairs[1]), np.maximum(pairs[0], pairs[1])
    key, inv = np.unique(lo * nN + hi, return_inverse=True)
    edges = np.stack([key // nN, key % nN])
    t2e = inv.reshape(3, nT)
    nE = edges.shape[1]
    t2f = np.zeros((14, nT), dtype=np.int64)
    t2f[:3] = t2e
    t2f[3] = np.arange(nT) + nE
    t2f[4:7] = t2e + nE + nT
    t2f[7] = np.arange(nT) + 2 * nE + nT
    t2f[8:11] = local + 2 * nE + 2 * nT
    t2f[11:14] = t2e + 2 * nE + 2 * nT + nN
    e2f = np.zeros((5, nE), dtype=np.int64)
    e2f[0] = np.arange(nE)
    e2f[1] = np.arange(nE) + nT + nE
    e2f[2] = np.arange(nE) + 2 * nE + 2 * nT + nN
    e2f[3:] = edges + 2 * nE + 2 * nT
    return PortSurface(node_ids, local, edges, t2e, t2f, e2f, 2 * nE + 2 * nT + nN + nE, 2 * nE + 2 * nT)


@dataclass
class PortModes:
    beta: np.ndarray            # propagation constants, ordered by closeness to the target
    eigenvalues: np.ndarray     # lambda = -beta^2
    modes: torch.Tensor         # (n_field, n_modes) complex, zero on PEC DOFs
    surface: PortSurface
    solve_ids: np.ndarray


@dataclass
class PortProblem:
    """The restricted 2-D port eigenproblem A x = lambda B x (dense, on the device)."""
    A: torch.Tensor             # (n, n) complex128, PEC DOFs removed
    B: torch.Tensor
    solve_ids: np.ndarray       # kept DOFs of the surface numbering
    surface: PortSurface
    target_kz: float            # the reference's default search target (or the one given)


def port_modes(field, er, ur, port_tags, basis, k0: float, pec_tags=(), target_kz: float | None = None,
               nmodes: int | None = None, face_block: bool = False,
               device: str | torch.device = "cuda") -> PortModes:
    """Modes of the port face ``port_tags`` at free-space wavenumber k0.

    Args:
        field: the 3-D Nedelec2-like field (``field.mesh`` with nodes, tris, edges,
            tri_to_edge, tri_to_tet, get_triangles).
        er, ur: (3, 3, n_tets) material tensors.
        basis: (3, 3) port frame (columns x, y, z; the reference's ``cs._basis``).
        pec_tags: face tags of the PEC boundary conditions.
        target_kz: the propagation constant searched around (the reference's
            default ermean*urmean*0.65*k0 when None, with the mean over the face).
        nmodes: keep at most this many modes (all that pass the filter when None).
        face_block: integrate the face-face entries of the transverse B block.  The
            reference leaves them zero (the default here, for parity), which puts the
            TE10 constant of a WR-90 port 4.9 % above the analytic value at any
            mesh size; with the block integrated it converges to it.
    """
    dev = torch.device(device)
    pp = port_problem(field, er, ur, port_tags, basis, k0, pec_tags, target_kz, face_block, device)
    As, Bs, S, solve_ids, target_kz = pp.A, pp.B, pp.surface, pp.solve_ids, pp.target_kz
    N = S.n_field
    sid = torch.as_tensor(solve_ids, device=dev)
    sigma = -float(target_kz) ** 2
    mu, vec = torch.linalg.eig(torch.linalg.solve(As - sigma * Bs, Bs))
    mu = mu.cpu().numpy()
    finite = np.abs(mu) > 1e-12 * np.abs(mu).max()
    lam = np.full(mu.shape, np.inf + 0j)
    lam[finite] = sigma + 1.0 / mu[finite]
    lr = lam.real
    keep = np.flatnonzero((lr <= -1) & (lr >= -(target_kz ** 2) * 8))
    beta = np.sqrt(-lam[keep])
    order = np.argsort(np.abs(beta - target_kz))
    keep, beta = keep[order], beta[order]
    if nmodes is not None:
        keep, beta = keep[:nmodes], beta[:nmodes]
    modes = torch.zeros((N, keep.size), dtype=torch.complex128, device=dev)
    modes[sid] = vec[:, torch.as_tensor(keep, device=dev)]
    return PortModes(beta, lam[keep], modes, S, solve_ids)


def port_problem(field, er, ur, port_tags, basis, k0: float, pec_tags=(), target_kz: float | None = None,
                 face_block: bool = False, device: str | torch.device = "cuda") -> PortProblem:
    """Steps 1-4 of ``port_modes``: the PEC-restricted dense A and B of the port face (the
    matrices the reference hands to ``SolveRoutine.eig``, emfreq3d.py:315)."""
    from .assembly import matinv_device
    dev = torch.device(device)
    m = field.mesh
    tri_ids = np.asarray(m.get_triangles(port_tags), dtype=np.int64)
    S = port_surface(m, tri_ids)
    nT = S.tris.shape[1]
    nodes2 = np.linalg.pinv(np.asarray(basis, dtype=float)) @ np.asarray(m.nodes)[:, S.node_ids]
    xy = np.ascontiguousarray(np.stack([nodes2[0][S.tris], nodes2[1][S.tris]]))            # (2, 3, nT)
    # local vertex positions of each edge inside its triangle (local_mapping)
    ev = S.edges[:, S.tri_to_edge]                                                         # (2, 3, nT)
    lem = np.argmax(S.tris[None, None, :, :] == ev[:, :, None, :], axis=2).astype(np.int32)   # (2, 3, nT)
    tet_of = np.asarray(m.tri_to_tet)[0, tri_ids]
    er_t = np.asarray(er)[:, :, tet_of]
    ur_t = np.asarray(ur)[:, :, tet_of]
    Ms9 = matinv_device(torch.as_tensor(np.ascontiguousarray(np.asarray(ur_t, dtype=np.complex128).reshape(9, nT)),
                                        device=dev))
    Mm9 = np.ascontiguousarray(np.asarray(er_t, dtype=np.complex128).reshape(9, nT))
    t = {k: torch.as_tensor(v, device=dev) for k, v in (("xy", xy), ("lem", np.ascontiguousarray(lem)),
                                                        ("Ms", Ms9), ("Mm", Mm9))}
    Ae = torch.empty((nT, 14, 14), dtype=torch.complex128, device=dev)
    Be = torch.empty((nT, 14, 14), dtype=torch.complex128, device=dev)
    with torch.cuda.device(dev):
        _lib.call("emg_port_element_matrices", nT, _vp(t["xy"]), _vp(t["lem"]), _vp(t["Ms"]), _vp(t["Mm"]),
                  ctypes.c_double(k0), int(bool(face_block)), _vp(Ae), _vp(Be),
                  ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream))
    f = torch.as_tensor(S.tri_to_field, device=dev)                                      # (14, nT)
    rows = f.T[:, :, None].expand(nT, 14, 14).reshape(-1)
    cols = f.T[:, None, :].expand(nT, 14, 14).reshape(-1)
    N = S.n_field

    def dense(vals):
        sp = torch.sparse_coo_tensor(torch.stack([rows, cols]), vals.reshape(-1), (N, N)).coalesce()
        return sp.to_dense()

    A, B = dense(Ae), dense(Be)
    # PEC: face edges on PEC triangles
    pec = np.zeros(N, dtype=bool)
    if len(pec_tags):
        ptri = np.asarray(m.get_triangles(list(pec_tags)), dtype=np.int64)
        e3 = np.unique(np.asarray(m.tri_to_edge)[:, ptri].ravel())
        ge = np.asarray(m.edges)[:, e3]
        pos = np.searchsorted(S.node_ids, ge)
        ok = (pos < S.node_ids.size).all(axis=0)
        ok[ok] &= (S.node_ids[pos[0, ok]] == ge[0, ok]) & (S.node_ids[pos[1, ok]] == ge[1, ok])
        nN = S.node_ids.size
        skey = S.edges[0] * nN + S.edges[1]
        lo, hi = np.minimum(pos[0, ok], pos[1, ok]), np.maximum(pos[0, ok], pos[1, ok])
        q = np.searchsorted(skey, lo * nN + hi)
        found = (q < skey.size) & (skey[np.minimum(q, skey.size - 1)] == lo * nN + hi)
        pec[S.edge_to_field[:, q[found]].ravel()] = True
        # PEC triangles that are face triangles: all their DOFs
        on_face = np.nonzero(np.isin(tri_ids, ptri))[0]
        if on_face.size:
            pec[S.tri_to_field[:, on_face].ravel()] = True
    solve_ids = np.flatnonzero(~pec)
    sid = torch.as_tensor(solve_ids, device=dev)
    As = A[sid][:, sid]
    Bs = B[sid][:, sid]
    if target_kz is None:
        d = np.concatenate([er_t[0, 0], er_t[1, 1], er_t[2, 2]])
        u = np.concatenate([ur_t[0, 0], ur_t[1, 1], ur_t[2, 2]])
        target_kz = float(np.mean(d.real) * np.mean(u.real) * 0.65 * k0)
    return PortProblem(As, Bs, solve_ids, S, float(target_kz))


def port_field(surface: PortSurface, nodes_local: np.ndarray, field, pts_local: np.ndarray, which: int = 0,
               urinv_diag: torch.Tensor | None = None, beta: float = 0.0) -> np.ndarray:
    """The port-mode field at points of the port plane (``emg_port_interp``): ``which`` 0
    gives E (ned2_tri_interp_full, fem/mth/tri.py:228-306), 1 the curl term of H
    (ned2_tri_interp_curl, fem/mth/tri.py:308-401, without its factor j/(omega mu0)),
    weighted by the diagonal of matinv(ur) per triangle (``urinv_diag``, (3, n_tris)
    complex on the device).  Local coordinates in, (3, npts) complex local components out."""
    field = torch.as_tensor(field)
    dev = field.device if field.is_cuda else torch.device("cuda")
    f = field.to(dev, torch.complex128).contiguous()
    xy = torch.as_tensor(np.ascontiguousarray(pts_local, dtype=np.float64), device=dev)
    nodes2 = torch.as_tensor(np.ascontiguousarray(nodes_local, dtype=np.float64), device=dev)
    tris = torch.as_tensor(np.ascontiguousarray(surface.tris, dtype=np.int32), device=dev)
    t2f = torch.as_tensor(np.ascontiguousarray(surface.tri_to_field, dtype=np.int32), device=dev)
    npts = int(xy.shape[1])
    out = torch.empty((3, npts), dtype=torch.complex128, device=dev)
    ud = None if urinv_diag is None else urinv_diag.to(dev, torch.complex128).contiguous()
    if which == 1 and ud is None:
        raise ValueError("port_field: the curl needs urinv_diag")
    with torch.cuda.device(dev):
        _lib.call("emg_port_interp", npts, _vp(xy), int(tris.shape[1]), _vp(tris), int(nodes2.shape[1]),
                  _vp(nodes2), _vp(t2f), _vp(f), _vp(ud) if ud is not None else None, ctypes.c_double(beta),
                  int(which), _vp(out), ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream))
    return out.cpu().numpy()
