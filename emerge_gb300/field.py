"""Field evaluation of second-order Nedelec solutions on the GPU.

``interpolate(field, solution, xs, ys, zs, tetids)`` is the counterpart of
``Nedelec2.interpolate`` / ``ned2_tet_interp`` (fem/elements/nedelec2.py:72-78,
fem/mth/tet.py:372-497): the E field of a solution vector at arbitrary points,
searched over the tets ``tetids`` (all tets by default), the last containing tet in
list order winning as in the reference, zero outside.  One CUDA thread per point
(emg_field_interp); the mesh arrays are uploaded once per field and cached on it.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib


def _vp(t) -> ctypes.c_void_p:
    return ctypes.c_void_p(t.data_ptr())


def _mesh_arrays(field, device):
    cache = getattr(field, "_emg_interp_mesh", None)
    if cache is None or cache[0] != device:
        m = field.mesh
        as_i32 = lambda a: torch.as_tensor(np.ascontiguousarray(np.asarray(a), dtype=np.int32), device=device)  # noqa: E731
        cache = (device, torch.as_tensor(np.ascontiguousarray(np.asarray(m.nodes), dtype=np.float64), device=device),
                 as_i32(m.tets), as_i32(m.edges), as_i32(m.tris), as_i32(field.tet_to_field))
        try:
            field._emg_interp_mesh = cache
        except AttributeError:
            pass
    return cache[1:]


def interpolate(field, solution, xs, ys, zs, tetids=None, device="cuda"):
    """(Ex, Ey, Ez) complex128 NumPy arrays of the solution's field at the points."""
    dev = torch.device(device)
    nodes, tets, edges, tris, t2f = _mesh_arrays(field, dev)
    pts = torch.as_tensor(np.ascontiguousarray(np.stack([np.ravel(xs), np.ravel(ys), np.ravel(zs)]),
                                               dtype=np.float64), device=dev)
    sol = solution if isinstance(solution, torch.Tensor) else torch.as_tensor(np.asarray(solution, dtype=np.complex128))
    sol = sol.to(dev, torch.complex128).contiguous()
    ids = torch.as_tensor(np.ascontiguousarray(np.arange(tets.shape[1]) if tetids is None else tetids, dtype=np.int32),
                          device=dev)
    n = pts.shape[1]
    E = torch.empty((3, n), dtype=torch.complex128, device=dev)
    _lib.call("emg_field_interp", n, _vp(pts), int(nodes.shape[1]), _vp(nodes), int(tets.shape[1]), _vp(tets),
              int(edges.shape[1]), _vp(edges), int(tris.shape[1]), _vp(tris), _vp(t2f), _vp(sol), int(ids.numel()),
              _vp(ids), _vp(E), ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream))
    E = E.cpu().numpy()
    return E[0], E[1], E[2]


def line_weights(field, points, dirs, tetids=None, device="cuda"):
    """Sparse linear functional of the field: (dofs, weights), each (n_points, 20), with
    sum(weights * x[dofs]) = sum_i dirs[:, i] . E_x(points[:, i]) for every solution x
    (emg_field_weights).  A voltage line integral is this with the line midpoints and
    steps (fem/physics/edm/emfreq3d.py:752-757).  Points in no tet of ``tetids`` get
    dof -1 and weight 0.  Returns CUDA tensors (int64 dofs, float64 weights)."""
    dev = torch.device(device)
    nodes, tets, edges, tris, t2f = _mesh_arrays(field, dev)
    pts = torch.as_tensor(np.ascontiguousarray(np.asarray(points, dtype=np.float64).reshape(3, -1)), device=dev)
    drs = torch.as_tensor(np.ascontiguousarray(np.asarray(dirs, dtype=np.float64).reshape(3, -1)), device=dev)
    ids = torch.as_tensor(np.ascontiguousarray(np.arange(tets.shape[1]) if tetids is None else tetids, dtype=np.int32),
                          device=dev)
    n = pts.shape[1]
    dofs = torch.empty((n, 20), dtype=torch.int32, device=dev)
    w = torch.empty((n, 20), dtype=torch.float64, device=dev)
    _lib.call("emg_field_weights", n, _vp(pts), _vp(drs), int(nodes.shape[1]), _vp(nodes), int(tets.shape[1]),
              _vp(tets), int(edges.shape[1]), _vp(edges), int(tris.shape[1]), _vp(tris), _vp(t2f), int(ids.numel()),
              _vp(ids), _vp(dofs), _vp(w), ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream))
    return dofs.to(torch.int64), w
