"""Oracle: CPU restatement of EMerge's FEM hot path (test infrastructure only).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline legs use
this package, and only as the checker or the timed CPU reference.  The product
package ``emerge_gb300`` never imports it.

``libned2_oracle.so`` (built from ned2_oracle.cpp by ``make -C oracle``)
restates the reference's element kernels and COO emission; COO -> CSR is
SciPy's ``coo_matrix(...).tocsr()``, exactly as the reference does
(fem/physics/edm/optimized_assembly.py:61-62).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

_f8p = ctypes.POINTER(ctypes.c_double)
_i8p = ctypes.POINTER(ctypes.c_int64)


def build() -> str:
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return os.path.join(_HERE, "libned2_oracle.so")


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "libned2_oracle.so")
        if not os.path.exists(path) or os.path.getmtime(path) < os.path.getmtime(os.path.join(_HERE, "ned2_oracle.cpp")):
            build()
        _LIB = ctypes.CDLL(path)
        L = _LIB
        L.orc_tet_stiff_mass.argtypes = [_f8p, _f8p, _i8p, _i8p, _f8p, _f8p, _f8p, _f8p]
        L.orc_matinv.argtypes = [_f8p, _f8p]
        L.orc_tet_coefficients_bcd.argtypes = [_f8p, _f8p, _f8p, _f8p, _f8p, _f8p, _f8p]
        L.orc_matrix_builder.argtypes = [_f8p, ctypes.c_int64, _i8p, ctypes.c_int64, _i8p, ctypes.c_int64, _i8p,
                                         ctypes.c_int64, _f8p, _i8p, _i8p, _f8p, _f8p, ctypes.c_int64,
                                         ctypes.c_int64, _f8p, _f8p, _i8p, _i8p]
        L.orc_tri_stiff_force.argtypes = [_f8p, ctypes.c_double, ctypes.c_double, _f8p, _f8p, ctypes.c_int, _f8p, _f8p]
        L.orc_tri_stiff.argtypes = [_f8p, _f8p, ctypes.c_double, ctypes.c_double, _f8p]
    return _LIB


def _p(a, t):
    return a.ctypes.data_as(t)


def _c(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


def tet_coefficients_bcd(verts):
    v = _c(verts, np.float64)
    b, c, d, V = (np.zeros(4), np.zeros(4), np.zeros(4), np.zeros(1))
    lib().orc_tet_coefficients_bcd(_p(v[0], _f8p), _p(v[1], _f8p), _p(v[2], _f8p), _p(b, _f8p), _p(c, _f8p),
                                   _p(d, _f8p), _p(V, _f8p))
    return b, c, d, V[0]


def matinv(s):
    s = _c(s, np.complex128)
    out = np.zeros((3, 3), dtype=np.complex128)
    lib().orc_matinv(_p(s.view(np.float64), _f8p), _p(out.view(np.float64), _f8p))
    return out


def tet_stiff_mass(verts, edge_lengths, lem, ltm, Ms, Mm):
    """ned2_tet_stiff_mass (fem/mth/tet.py:854-1088) -> (D, F) 20x20 complex."""
    v = _c(verts, np.float64)
    el = _c(edge_lengths, np.float64)
    lem = _c(lem, np.int64)
    ltm = _c(ltm, np.int64)
    Ms = _c(Ms, np.complex128)
    Mm = _c(Mm, np.complex128)
    D = np.zeros((20, 20), dtype=np.complex128)
    F = np.zeros((20, 20), dtype=np.complex128)
    lib().orc_tet_stiff_mass(_p(v, _f8p), _p(el, _f8p), _p(lem, _i8p), _p(ltm, _i8p), _p(Ms.view(np.float64), _f8p),
                             _p(Mm.view(np.float64), _f8p), _p(D.view(np.float64), _f8p), _p(F.view(np.float64), _f8p))
    return D, F


def matrix_builder(field, er, ur, t0: int = 0, t1: int | None = None):
    """_matrix_builder (fem/physics/edm/optimized_assembly.py:76-116) over tets [t0, t1).

    Returns (dataE, dataB, rows, cols) with 400 entries per tet, in the reference's order.
    """
    m = field.mesh
    nT = m.tets.shape[1]
    t1 = nT if t1 is None else t1
    n = (t1 - t0) * 400
    nodes = _c(m.nodes, np.float64)
    tets = _c(m.tets, np.int64)
    tris = _c(m.tris, np.int64)
    edges = _c(m.edges, np.int64)
    el = _c(m.edge_lengths, np.float64)
    t2f = _c(field.tet_to_field, np.int64)
    t2e = _c(m.tet_to_edge, np.int64)
    ur = _c(ur, np.complex128)
    er = _c(er, np.complex128)
    dE = np.empty(n, dtype=np.complex128)
    dB = np.empty(n, dtype=np.complex128)
    rows = np.empty(n, dtype=np.int64)
    cols = np.empty(n, dtype=np.int64)
    lib().orc_matrix_builder(_p(nodes, _f8p), nodes.shape[1], _p(tets, _i8p), nT, _p(tris, _i8p), tris.shape[1],
                             _p(edges, _i8p), edges.shape[1], _p(el, _f8p), _p(t2f, _i8p), _p(t2e, _i8p),
                             _p(ur.view(np.float64), _f8p), _p(er.view(np.float64), _f8p), t0, t1,
                             _p(dE.view(np.float64), _f8p), _p(dB.view(np.float64), _f8p), _p(rows, _i8p),
                             _p(cols, _i8p))
    return dE, dB, rows, cols


def tet_mass_stiffness_matrices(field, er, ur):
    """tet_mass_stiffness_matrices (fem/physics/edm/optimized_assembly.py:43-64) -> (E, B) CSR."""
    from scipy.sparse import coo_matrix
    m = field.mesh
    N = 2 * m.edges.shape[1] + 2 * m.tris.shape[1]
    dE, dB, rows, cols = matrix_builder(field, er, ur)
    E = coo_matrix((dE, (rows, cols)), shape=(N, N)).tocsr()
    B = coo_matrix((dB, (rows, cols)), shape=(N, N)).tocsr()
    return E, B


def rows_csr(field, er, ur, rows):
    """Rows ``rows`` (ascending DOF ids) of the reference's E and B as CSR matrices of shape
    (len(rows), N), without assembling the whole mesh.

    Only the tets that touch one of the rows contribute to them; those tets run through
    ``matrix_builder`` in ascending tet order, so every entry receives its contributions
    in the same order as in the full COO array, and SciPy's ``tocsr`` sums them as the
    reference's whole-mesh ``tocsr`` does (fem/physics/edm/optimized_assembly.py:61-62).
    """
    import types
    from scipy.sparse import coo_matrix
    m = field.mesh
    rows = np.asarray(rows, dtype=np.int64)
    N = 2 * m.edges.shape[1] + 2 * m.tris.shape[1]
    t2f = np.asarray(field.tet_to_field, dtype=np.int64)
    touch = np.isin(t2f, rows).any(axis=0)
    sel = np.flatnonzero(touch)
    sub_mesh = types.SimpleNamespace(nodes=m.nodes, tets=np.asarray(m.tets)[:, sel], tris=m.tris, edges=m.edges,
                                     edge_lengths=m.edge_lengths, tet_to_edge=np.asarray(m.tet_to_edge)[:, sel])
    sub = types.SimpleNamespace(mesh=sub_mesh, tet_to_field=t2f[:, sel])
    dE, dB, r, c = matrix_builder(sub, np.asarray(er)[:, :, sel], np.asarray(ur)[:, :, sel])
    local = np.searchsorted(rows, r)
    keep = (local < len(rows)) & (rows[np.minimum(local, len(rows) - 1)] == r)
    shape = (len(rows), N)
    E = coo_matrix((dE[keep], (local[keep], c[keep])), shape=shape).tocsr()
    B = coo_matrix((dB[keep], (local[keep], c[keep])), shape=shape).tocsr()
    return E, B, len(sel)


def tri_stiff_force(lcs_vertices, gamma, Uinc, DPTs):
    """ned2_tri_stiff_force (fem/mth/tri.py:575-695) -> (B 8x8, b 8)."""
    lv = _c(lcs_vertices, np.float64)
    U = _c(Uinc, np.complex128)
    P = _c(DPTs, np.float64)
    B = np.zeros((8, 8), dtype=np.complex128)
    b = np.zeros(8, dtype=np.complex128)
    g = complex(gamma)
    lib().orc_tri_stiff_force(_p(lv, _f8p), g.real, g.imag, _p(U.view(np.float64), _f8p), _p(P, _f8p),
                              P.shape[1], _p(B.view(np.float64), _f8p), _p(b.view(np.float64), _f8p))
    return B, b


def tri_stiff(vertices, edge_lengths, gamma):
    """ned2_tri_stiff (fem/mth/tri.py:697-797) -> B 8x8."""
    v = _c(vertices, np.float64)
    el = _c(edge_lengths, np.float64)
    B = np.zeros((8, 8), dtype=np.complex128)
    g = complex(gamma)
    lib().orc_tri_stiff(_p(v, _f8p), _p(el, _f8p), g.real, g.imag, _p(B.view(np.float64), _f8p))
    return B
