"""GPU mesh topology: the edge/face arrays of ``Mesh3D.update`` and the Nédélec-2 DOF map.

``Mesh3D.update`` (fem/mesh3d.py:224-355) builds the edges, faces and their
incidence maps with Python loops and dicts over the tets, and
``Nedelec2.__init__`` (fem/elements/nedelec2.py:32-62) the tet -> DOF map. At
millions of tets those loops take minutes. ``build_topology`` does the same with
radix sorts on the GPU (``emg_topology_create``); ``TetMesh(..., device="cuda")``
uses it. Numbering is ascending vertex-tuple order, bitwise equal to the host
builder in ``mesh.py``.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib


def _vp(t: torch.Tensor) -> ctypes.c_void_p:
    return ctypes.c_void_p(t.data_ptr())


def _stream() -> ctypes.c_void_p:
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def build_topology(nodes: np.ndarray, tets: np.ndarray, device: str | torch.device = "cuda",
                   keep_on_device: bool = False) -> dict:
    """Edges, faces, incidence maps, tet_to_field and edge lengths of a tet mesh.

    Args:
        nodes: (3, nN) float64 vertex coordinates (NumPy, or a torch tensor).
        tets: (4, nT) vertex indices (NumPy, or a torch tensor; int32 on the device).
        keep_on_device: return torch CUDA tensors (int32 / float64) instead of
            host int64 / float64 arrays.

    Returns a dict with ``edges (2,nE)``, ``tris (3,nTri)``, ``tet_to_edge (6,nT)``,
    ``tet_to_tri (4,nT)``, ``tri_to_edge (3,nTri)``, ``tri_to_tet (2,nTri)``,
    ``tet_to_field (20,nT)`` and ``edge_lengths (nE,)``.
    """
    _lib.load()
    dev = torch.device(device)
    if isinstance(nodes, torch.Tensor):
        nodes_d = nodes.to(device=dev, dtype=torch.float64).contiguous()
    else:
        nodes_d = torch.as_tensor(np.ascontiguousarray(nodes, dtype=np.float64), device=dev)
    if isinstance(tets, torch.Tensor):
        tets_d = tets.to(device=dev, dtype=torch.int32).contiguous()
    else:
        tets_d = torch.as_tensor(np.ascontiguousarray(tets, dtype=np.int32), device=dev)
    nN, nT = int(nodes_d.shape[1]), int(tets_d.shape[1])
    h = ctypes.c_void_p()
    with torch.cuda.device(dev):
        _lib.call("emg_topology_create", nN, nT, _vp(tets_d), _stream(), ctypes.byref(h))
        try:
            ne, nf = ctypes.c_int64(), ctypes.c_int64()
            _lib.call("emg_topology_sizes", h, ctypes.byref(ne), ctypes.byref(nf))
            nE, nTri = ne.value, nf.value
            i32 = dict(dtype=torch.int32, device=dev)
            out = {"edges": torch.empty((2, nE), **i32), "tris": torch.empty((3, nTri), **i32),
                   "tet_to_edge": torch.empty((6, nT), **i32), "tet_to_tri": torch.empty((4, nT), **i32),
                   "tri_to_edge": torch.empty((3, nTri), **i32), "tri_to_tet": torch.empty((2, nTri), **i32),
                   "tet_to_field": torch.empty((20, nT), **i32)}
            _lib.call("emg_topology_get", h, *[_vp(out[k]) for k in ("edges", "tris", "tet_to_edge", "tet_to_tri",
                                                                      "tri_to_edge", "tri_to_tet", "tet_to_field")],
                      _stream())
            out["edge_lengths"] = torch.empty(nE, dtype=torch.float64, device=dev)
            _lib.call("emg_edge_lengths", nN, _vp(nodes_d), nE, _vp(out["edges"]), _vp(out["edge_lengths"]),
                      _stream())
            torch.cuda.current_stream().synchronize()
        finally:
            _lib.load().emg_topology_destroy(h)
    if keep_on_device:
        return out
    host = {k: v.cpu().numpy() for k, v in out.items()}
    for k in host:
        if k != "edge_lengths":
            host[k] = host[k].astype(np.int64)
    return host
