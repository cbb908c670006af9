"""Oracle for the GPU Stratton-Chu far field (test infrastructure only).

NumPy FP64 restatement of fem/physics/edm/sc.py:

- ``surface_weights`` is the weight loop of ``stratton_chu`` (sc.py:149-165): every
  surface triangle adds n·area/3 to each of its three edges, in triangle order.
- ``stratton_chu_ff`` follows sc.py:41-140:
  - sources with |E| <= max|E| · 1e-3 are dropped;
  - the direction is r = (cos θ cos φ, cos θ sin φ, sin θ);
  - per source, G = exp(j k0 r·v) and ie = (n×E − Z0 r×(n×H))·G;
  - E_ff = Σ Q r×ie with Q = −j k0/(4π), and H_ff = r×E_ff / Z0.
"""
from __future__ import annotations

import numpy as np

Z0 = 376.73031366857
LR = 0.001


def surface_weights(n_edges, tri_to_edge, normals, areas) -> np.ndarray:
    """(3, n_edges) float32 weights, accumulated tri by tri as sc.py:159-165 does."""
    wns = np.zeros((3, n_edges), dtype=np.float32)
    for i in range(tri_to_edge.shape[1]):
        v = normals[:, i] * areas[i] / 3
        for e in tri_to_edge[:, i]:
            wns[:, e] += v
    return wns


def stratton_chu_ff(Ein, Hin, vis, wns, theta, phi, k0):
    """(Eout, Hout) complex (3, n_dirs), in FP64 from the FP32/complex64 inputs."""
    E = np.asarray(Ein, dtype=np.complex64).astype(np.complex128)
    H = np.asarray(Hin, dtype=np.complex64).astype(np.complex128)
    v = np.asarray(vis, dtype=np.float32).astype(np.float64)
    n = np.asarray(wns, dtype=np.float32).astype(np.float64)
    th = np.asarray(theta, dtype=np.float32).astype(np.float64)
    ph = np.asarray(phi, dtype=np.float32).astype(np.float64)
    k = float(np.float32(k0))
    Emag = np.sqrt(np.abs(E[0]) ** 2 + np.abs(E[1]) ** 2 + np.abs(E[2]) ** 2)
    keep = Emag > np.max(Emag) * LR
    E, H, v, n = E[:, keep], H[:, keep], v[:, keep], n[:, keep]
    r = np.stack([np.cos(th) * np.cos(ph), np.cos(th) * np.sin(ph), np.sin(th)])      # (3, N)
    nxe = np.cross(n.T, E.T).T                                                       # (3, M)
    nxh = np.cross(n.T, H.T).T
    Q = -1j * k / (4 * np.pi)
    out = np.zeros((3, r.shape[1]), dtype=np.complex128)
    for j0 in range(0, v.shape[1], 2048):
        sl = slice(j0, j0 + 2048)
        G = np.exp(1j * k * (r.T @ v[:, sl]))                                          # (N, m)
        # r x (n x H) per (direction, source)
        a = nxh[:, sl]
        rx, ry, rz = r[0][:, None], r[1][:, None], r[2][:, None]
        rh = [ry * a[2] - rz * a[1], rz * a[0] - rx * a[2], rx * a[1] - ry * a[0]]
        ie = [(nxe[c, sl][None, :] - Z0 * rh[c]) * G for c in range(3)]
        out[0] += Q * np.sum(ry * ie[2] - rz * ie[1], axis=1)
        out[1] += Q * np.sum(rz * ie[0] - rx * ie[2], axis=1)
        out[2] += Q * np.sum(rx * ie[1] - ry * ie[0], axis=1)
    Hout = np.stack([r[1] * out[2] - r[2] * out[1], r[2] * out[0] - r[0] * out[2],
                     r[0] * out[1] - r[1] * out[0]]) / Z0
    return out, Hout
