"""Oracle for the GPU port-mode element matrices (test infrastructure only).

NumPy FP64 restatement of generalized_matrix_GQ
(fem/physics/edm/nedeleclegrange2.py:224-382): the 14 x 14 element matrices of
the 2-D waveguide-port eigenproblem A x = lambda B x (lambda = -beta^2) on one
triangle, with second-order Nedelec transverse functions (DOFs 0-7) and
second-order Lagrange longitudinal functions (DOFs 8-13).

Notation: lambda_i = a_i + b_i x + c_i y are the barycentric functions (the
tri_coefficients of nedeleclegrange2.py:192-214 over 2 area, sign-corrected);
for an edge (p, q) (its local vertices from the local edge map):
    N1 = (grad l_p l_q - grad l_q l_p) l_p,   N2 = (...) l_q,
    curl N1 = 3 l_p (b_q c_p - b_p c_q),      curl N2 = 3 l_q (b_q c_p - b_p c_q),
    L_edge = 4 l_p l_q;
for the face (vertices 0, 1, 2 in triangle order):
    F1 = -(grad l_0 l_2 - grad l_2 l_0) l_1,  F2 = (grad l_0 l_1 - grad l_1 l_0) l_2;
for vertex i: L_i = 2 l_i^2 - l_i.
Blocks (6-point rule of the module's DPTS, times the area):
    Att = curl.Ms_zz.curl, Btt = N.Mm_t.N, Dtt = N.Ms_t.N, Dzt = grad L.Ms_t.N,
    Dzz = grad L.Ms_t.grad L - k0^2 L.Mm_zz.L,
    A[:8, :8] = Att - k0^2 Btt,  B = [[Dtt, Dzt^T], [Dzt, Dzz]],
each scaled by the lengths of the DOFs' edges (face DOFs: |v0 v2| and |v0 v1|).
The reference's quirks are kept: the face-edge entries of Att, Btt and Dtt are
mirrored from the edge-face ones (not recomputed), and the face-face entries of
Dtt stay zero.
"""
from __future__ import annotations

import numpy as np

# 6-point rule: weights (row 0) and barycentric coordinates (rows 1-3), as written in
# fem/physics/edm/nedeleclegrange2.py:218-221
DPTS = np.array([[0.22338159, 0.22338159, 0.22338159, 0.10995174, 0.10995174, 0.10995174],
                 [0.10810302, 0.44594849, 0.44594849, 0.81684757, 0.09157621, 0.09157621],
                 [0.44594849, 0.44594849, 0.10810302, 0.09157621, 0.09157621, 0.81684757],
                 [0.44594849, 0.10810302, 0.44594849, 0.09157621, 0.81684757, 0.09157621]])


def element_matrices(verts, lem, Ms, Mm, k0, face_block=False):
    """(A, B) 14x14 complex of one triangle: verts (2, 3), lem (2, 3) local edge map.
    face_block: integrate the face-face entries of Dtt instead of the reference's zeros."""
    x, y = np.asarray(verts, dtype=float)[0], np.asarray(verts, dtype=float)[1]
    W = DPTS[0]
    xs = x[0] * DPTS[1] + x[1] * DPTS[2] + x[2] * DPTS[3]
    ys = y[0] * DPTS[1] + y[1] * DPTS[2] + y[2] * DPTS[3]
    a = np.array([x[1] * y[2] - y[1] * x[2], x[2] * y[0] - y[2] * x[0], x[0] * y[1] - y[0] * x[1]])
    b = np.array([y[1] - y[2], y[2] - y[0], y[0] - y[1]])
    c = np.array([x[2] - x[1], x[0] - x[2], x[1] - x[0]])
    sA = 0.5 * ((x[0] - x[2]) * (y[1] - y[0]) - (x[0] - x[1]) * (y[2] - y[0]))
    sg = np.sign(sA)
    area = abs(sA)
    a, b, c = a * sg / (2 * area), b * sg / (2 * area), c * sg / (2 * area)
    lam = a[:, None] + b[:, None] * xs[None, :] + c[:, None] * ys[None, :]          # (3, q)
    Ms = np.asarray(Ms, dtype=np.complex128)
    Mm = np.asarray(Mm, dtype=np.complex128)
    Msz, Mmz, Mst, Mmt = Ms[2, 2], Mm[2, 2], Ms[:2, :2], Mm[:2, :2]

    def whit(p, q):                     # grad l_p l_q - grad l_q l_p, (2, q)
        return np.array([b[p] * lam[q] - b[q] * lam[p], c[p] * lam[q] - c[q] * lam[p]])

    edges = [tuple(int(v) for v in lem[:, e]) for e in range(3)]
    N = [None] * 8                       # transverse functions (2, q)
    C = [None] * 8                       # their curls (q,)
    for e, (p, q) in enumerate(edges):
        w = whit(p, q)
        rot = b[q] * c[p] - b[p] * c[q]
        N[e], N[4 + e] = w * lam[p], w * lam[q]
        C[e], C[4 + e] = 3 * lam[p] * rot, 3 * lam[q] * rot
    N[3] = -whit(0, 2) * lam[1]
    N[7] = whit(0, 1) * lam[2]
    C[3] = -b[1] * (c[0] * lam[2] - c[2] * lam[0]) + c[1] * (b[0] * lam[2] - b[2] * lam[0]) + \
        2 * (b[0] * c[2] - b[2] * c[0]) * lam[1]
    C[7] = b[2] * (c[0] * lam[1] - c[1] * lam[0]) - c[2] * (b[0] * lam[1] - b[1] * lam[0]) - \
        2 * (b[0] * c[1] - b[1] * c[0]) * lam[2]
    Lz = [2 * lam[i] ** 2 - lam[i] for i in range(3)] + [4 * lam[p] * lam[q] for p, q in edges]
    Gz = [np.array([b[i] * (4 * lam[i] - 1), c[i] * (4 * lam[i] - 1)]) for i in range(3)] + \
         [4 * np.array([b[p] * lam[q] + b[q] * lam[p], c[p] * lam[q] + c[q] * lam[p]]) for p, q in edges]

    def dot(u, M, v):                    # sum_q W (u . M v)
        return np.sum(W * np.sum(u * (M @ v), axis=0))

    Att = np.zeros((8, 8), dtype=np.complex128)
    Btt = np.zeros((8, 8), dtype=np.complex128)
    Dtt = np.zeros((8, 8), dtype=np.complex128)
    Dzt = np.zeros((6, 8), dtype=np.complex128)
    Dzz = np.zeros((6, 6), dtype=np.complex128)
    tt = [0, 1, 2, 4, 5, 6]              # edge DOFs
    for i in tt:
        for j in tt:
            Att[i, j] = np.sum(W * C[i] * Msz * C[j])
            Btt[i, j] = dot(N[i], Mmt, N[j])
            Dtt[i, j] = dot(N[i], Mst, N[j])
        for j in (3, 7):                 # edge rows, face columns; mirrored below
            Att[i, j] = np.sum(W * C[i] * Msz * C[j])
            Btt[i, j] = dot(N[i], Mmt, N[j])
            Dtt[i, j] = dot(N[i], Mst, N[j])
            Att[j, i], Btt[j, i], Dtt[j, i] = Att[i, j], Btt[i, j], Dtt[i, j]
    for i in (3, 7):
        for j in (3, 7):
            Att[i, j] = np.sum(W * C[i] * Msz * C[j])
            Btt[i, j] = dot(N[i], Mmt, N[j])
            if face_block:
                Dtt[i, j] = dot(N[i], Mst, N[j])
    for k in range(6):
        for j in range(8):
            Dzt[k, j] = dot(Gz[k], Mst, N[j])
        for l in range(6):
            Dzz[k, l] = dot(Gz[k], Mst, Gz[l]) - k0 ** 2 * np.sum(W * Lz[k] * Mmz * Lz[l])
    A = np.zeros((14, 14), dtype=np.complex128)
    B = np.zeros((14, 14), dtype=np.complex128)
    A[:8, :8] = Att - k0 ** 2 * Btt
    B[:8, :8] = Dtt
    B[8:, :8] = Dzt
    B[:8, 8:] = Dzt.T
    B[8:, 8:] = Dzz
    Dv = lambda i, j: np.hypot(x[i] - x[j], y[i] - y[j])               # noqa: E731
    Ls = np.ones(14)
    for e, (p, q) in enumerate(edges):
        Ls[e] = Ls[4 + e] = Dv(p, q)
    Ls[3], Ls[7] = Dv(0, 2), Dv(0, 1)
    S = np.outer(Ls, Ls) * area
    return S * A, S * B
