"""GPU drop-in for EMerge's Stratton-Chu far-field transform.

``stratton_chu(Ein, Hin, mesh, theta, phi, k0)`` has the signature and return
value of fem/physics/edm/sc.py:143-180: the far-field E and H (complex128,
(3, n_directions)) radiated by the surface fields Ein, Hin sampled at the edge
centres of ``mesh``. ``mesh`` is any object with the SurfaceMesh attributes
the reference reads: ``n_tris``, ``tri_to_edge (3, nTri)``, ``normals (3, nTri)``,
``areas (nTri,)`` and ``edge_centers (3, nE)``. Directions are elevation ``theta``
and azimuth ``phi``: r = (cos θ cos φ, cos θ sin φ, sin θ).

The source weights n·area/3 are accumulated on the host exactly as the
reference does (sc.py:159-165). The transform runs on the GPU
(``emg_stratton_chu``), with FP32 sources and FP32 accumulation per chunk of 512
sources, then FP64 across chunks.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib


def _vp(t: torch.Tensor) -> ctypes.c_void_p:
    return ctypes.c_void_p(t.data_ptr())


def surface_weights(mesh) -> np.ndarray:
    """(3, nE) float32: every triangle adds n·area/3 to its three edges, in triangle order."""
    t2e = np.asarray(mesh.tri_to_edge, dtype=np.int64)
    nrm = np.asarray(mesh.normals, dtype=np.float64)
    area = np.asarray(mesh.areas, dtype=np.float64)
    ne = np.asarray(mesh.edge_centers).shape[1]
    wns = np.zeros((3, ne), dtype=np.float32)
    vals = nrm * area[None, :] / 3                                   # (3, nTri), as n*areas[i]/3
    idx = t2e.T.ravel()                                              # tri-major, edge slots in order
    for c in range(3):
        np.add.at(wns[c], idx, np.repeat(vals[c], 3))
    return wns


def stratton_chu(Ein, Hin, mesh, theta, phi, k0: float, device: str | torch.device = "cuda"):
    """Drop-in for fem/physics/edm/sc.py:143-180 -> (Eout, Hout) complex128 (3, n_dirs)."""
    _lib.load()
    dev = torch.device(device)
    E = np.ascontiguousarray(np.asarray(Ein).astype(np.complex64))
    H = np.ascontiguousarray(np.asarray(Hin).astype(np.complex64))
    vis = np.ascontiguousarray(np.asarray(mesh.edge_centers, dtype=np.float32))
    wns = surface_weights(mesh)
    th = np.ascontiguousarray(np.asarray(theta, dtype=np.float32).ravel())
    ph = np.ascontiguousarray(np.asarray(phi, dtype=np.float32).ravel())
    if E.shape != H.shape or E.shape[0] != 3 or E.shape[1] != vis.shape[1] or th.shape != ph.shape:
        raise ValueError("Ein, Hin must be (3, n_edges) like mesh.edge_centers; theta and phi of equal length")
    ns, nd = E.shape[1], th.size
    t = {k: torch.as_tensor(v, device=dev) for k, v in
         (("E", E), ("H", H), ("vis", vis), ("wns", wns), ("th", th), ("ph", ph))}
    Eout = torch.empty((3, nd), dtype=torch.complex128, device=dev)
    Hout = torch.empty((3, nd), dtype=torch.complex128, device=dev)
    with torch.cuda.device(dev):
        _lib.call("emg_stratton_chu", ns, _vp(t["E"]), _vp(t["H"]), _vp(t["vis"]), _vp(t["wns"]), nd, _vp(t["th"]),
                  _vp(t["ph"]), ctypes.c_float(np.float32(k0)), _vp(Eout), _vp(Hout),
                  ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    return Eout.cpu().numpy(), Hout.cpu().numpy()
