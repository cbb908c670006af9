"""Oracle for the GPU field interpolation (test infrastructure only).

NumPy FP64 restatement of ned2_tet_interp (fem/mth/tet.py:372-497): the
second-order Nedelec field of a solution vector at arbitrary points.

- Location: a point belongs to a tet of ``tetids`` when its local coordinates
  (the inverse of the edge basis [v2-v1, v3-v1, v4-v1] applied to p - v1) satisfy
  xi >= -1e-6 and sum(xi) <= 1 + 1e-8. Tets are scanned in order, so the last
  containing tet wins; a point in none gets 0.
- Field: with the barycentric numerators A_i = a_i + b_i x + c_i y + d_i z
  (= det(P) lambda_i) and 216 V^3 = |det(P)|^3, the formulas are
  - edge (vertices 1, 2; length L):
    L (e1 A1 + e2 A2) (g1 A2 - g2 A1) / (216 V^3) for g = b, c, d;
  - face (vertices 1, 2, 3; L1 = |v1 v3|, L2 = |v1 v2|):
    (-e1 L1 (g1 A3 - g3 A1) A2 + e2 L2 (g1 A2 - g2 A1) A3) / (216 V^3).
- Vertex order of an edge or face is that of the mesh's edges/tris arrays.
"""
from __future__ import annotations

import numpy as np


def _local(tet_vertices: np.ndarray, ids: np.ndarray) -> np.ndarray:
    """Local indices (0..3) inside the tet of every global vertex id in ``ids``."""
    out = np.empty(ids.shape, dtype=np.int64)
    for r in range(ids.shape[0]):
        for c in range(ids.shape[1]):
            out[r, c] = int(np.flatnonzero(tet_vertices == ids[r, c])[0])
    return out


def interpolate(points, solution, tets, tris, edges, nodes, tet_to_field, tetids):
    """(Ex, Ey, Ez) complex at the points (3, n)."""
    pts = np.asarray(points, dtype=np.float64)
    n = pts.shape[1]
    E = np.zeros((3, n), dtype=np.complex128)
    nE = edges.shape[1]
    for t in np.asarray(tetids, dtype=np.int64):
        tv = tets[:, t]
        V = nodes[:, tv]                                    # (3, 4)
        Bm = np.stack([V[:, 1] - V[:, 0], V[:, 2] - V[:, 0], V[:, 3] - V[:, 0]], axis=1)
        xi = np.linalg.inv(Bm) @ (pts - V[:, :1])
        inside = (xi.sum(axis=0) <= 1.00000001) & np.all(xi >= -1e-6, axis=0)
        if not inside.any():
            continue
        P = np.concatenate([np.ones((4, 1)), V.T], axis=1)  # rows (1, x_j, y_j, z_j)
        detP = np.linalg.det(P)
        C = detP * np.linalg.inv(P)                         # column i: (a_i, b_i, c_i, d_i)
        q = pts[:, inside]
        A = C[0][:, None] + C[1][:, None] * q[0] + C[2][:, None] * q[1] + C[3][:, None] * q[2]   # (4, m)
        den = abs(detP) ** 3
        f = tet_to_field[:, t]
        sol = solution[f]
        le = _local(tv, edges[:, f[0:6]])
        lt = _local(tv, tris[:, f[6:10] - nE])
        out = np.zeros((3, q.shape[1]), dtype=np.complex128)
        for ie in range(6):
            i1, i2 = le[:, ie]
            L = np.linalg.norm(V[:, i1] - V[:, i2])
            s = sol[ie] * A[i1] + sol[10 + ie] * A[i2]
            for d in range(3):
                out[d] += L * s * (C[1 + d, i1] * A[i2] - C[1 + d, i2] * A[i1]) / den
        for jf in range(4):
            i1, i2, i3 = lt[:, jf]
            L1 = np.linalg.norm(V[:, i1] - V[:, i3])
            L2 = np.linalg.norm(V[:, i1] - V[:, i2])
            e1, e2 = sol[6 + jf], sol[16 + jf]
            for d in range(3):
                g1, g2, g3 = C[1 + d, i1], C[1 + d, i2], C[1 + d, i3]
                out[d] += (-e1 * L1 * (g1 * A[i3] - g3 * A[i1]) * A[i2]
                           + e2 * L2 * (g1 * A[i2] - g2 * A[i1]) * A[i3]) / den
        E[:, inside] = out
    return E[0], E[1], E[2]
