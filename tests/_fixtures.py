"""Helpers that turn the golden .npz fixtures into Nedelec2-like objects."""
from __future__ import annotations

import os
import types

import numpy as np

from conftest import GOLDEN


def load(name: str):
    return np.load(os.path.join(GOLDEN, name))


def field_from(z) -> types.SimpleNamespace:
    """A Nedelec2-like view (``field.mesh.*``, ``field.tet_to_field``) of fixture arrays."""
    i8 = lambda k: np.asarray(z[k], dtype=np.int64)  # noqa: E731
    mesh = types.SimpleNamespace(nodes=np.asarray(z["nodes"]), tets=i8("tets"), tris=i8("tris"), edges=i8("edges"),
                                 edge_lengths=np.asarray(z["edge_lengths"]), tet_to_edge=i8("tet_to_edge"),
                                 tet_to_tri=i8("tet_to_tri"), tri_to_edge=i8("tri_to_edge"))
    if "tri_to_tet" in z:
        mesh.tri_to_tet = i8("tri_to_tet")
    mesh.n_tets = mesh.tets.shape[1]
    mesh.n_edges = mesh.edges.shape[1]
    mesh.n_tris = mesh.tris.shape[1]
    f = types.SimpleNamespace(mesh=mesh, tet_to_field=i8("tet_to_field"))
    f.n_field = 2 * mesh.n_edges + 2 * mesh.n_tris
    nE, nF = mesh.n_edges, mesh.n_tris
    f.edge_to_field = np.stack([np.arange(nE), np.arange(nE) + nF + nE]).astype(np.int64)
    if "tri_to_field" in z:
        f.tri_to_field = i8("tri_to_field")
    return f


def waveguide_field_and_bcs(z):
    """The WR-90 fixture as a field plus project BC objects mirroring the reference run."""
    from emerge_gb300 import bc as pbc
    from emerge_gb300 import mesh as pm
    field = field_from(z)
    a, b, L = (float(v) for v in z["dims"])
    tag_tris = {(pm.FACE_YMIN,): z["port_tris_1"], (pm.FACE_YMAX,): z["port_tris_2"],
                (pm.FACE_XMIN, pm.FACE_XMAX, pm.FACE_ZMIN, pm.FACE_ZMAX): z["pec_tris"]}
    field.mesh.get_triangles = lambda tags: np.asarray(tag_tris[tuple(tags)], dtype=np.int64)
    p1 = pbc.RectangularWaveguide([pm.FACE_YMIN], 1, pbc.CoordinateSystem([1.0, 0, 0], [0, 0, 1.0], [0, -1.0, 0],
                                                                        [a / 2, 0.0, b / 2]), (a, b))
    p2 = pbc.RectangularWaveguide([pm.FACE_YMAX], 2, pbc.CoordinateSystem([-1.0, 0, 0], [0, 0, 1.0], [0, 1.0, 0],
                                                                        [a / 2, L, b / 2]), (a, b))
    pec = pbc.PEC([pm.FACE_XMIN, pm.FACE_XMAX, pm.FACE_ZMIN, pm.FACE_ZMAX])
    return field, [pec, p1, p2]


def csr_from(z, prefix: str):
    from scipy.sparse import csr_matrix
    ip = z[prefix + "_indptr"]
    n = len(ip) - 1
    return csr_matrix((z[prefix + "_data"], z[prefix + "_indices"], ip), shape=(n, n))


def rel_to_rowmax(A, R) -> float:
    """max |A - R| per entry relative to the largest |R| of its row (same pattern required)."""
    assert np.array_equal(A.indptr, R.indptr) and np.array_equal(A.indices, R.indices)
    if R.nnz == 0:
        return 0.0
    ip = R.indptr
    nz_rows = np.diff(ip) > 0
    rowmax = np.zeros(len(ip) - 1)
    rowmax[nz_rows] = np.maximum.reduceat(np.abs(R.data), ip[:-1][nz_rows])
    scale = np.repeat(rowmax, np.diff(ip))
    scale[scale == 0] = 1.0
    return float(np.max(np.abs(A.data - R.data) / scale))
