"""Import shims that let the EMerge reference run in this container.

Used only by ``make_golden.py`` (fixture generation, run where the reference
checkout exists).  The reference needs numba, numba_progress, loguru, gmsh and
pypardiso, none of which is installed; this module registers stand-ins:

* ``numba``: ``njit``/``jit`` return the function unchanged, ``prange`` is
  ``range`` and the type objects accept any indexing/call, so the Numba kernels
  run as plain Python with IEEE double arithmetic.
* ``numba_progress``: a no-op progress bar.
* ``loguru``: a silent logger.
* ``gmsh``: serves one project mesh (nodes, tets, tagged boundary triangles,
  volumes) through the handful of ``gmsh.model.mesh`` calls ``Mesh3D`` makes.
* ``pypardiso``: not needed (SuperLU is used), registered empty.

The ``fem`` packages are registered as namespace modules so that
``fem/__init__.py`` (which imports the CAD and plotting stacks) is skipped.
"""
from __future__ import annotations

import os
import sys
import types

import numpy as np

# Root of the EMerge checkout (the directory holding ``fem/``): set by
# ``make_golden.py --ref PATH`` or the EMERGE_REF_ROOT environment variable.
REF_ROOT = os.environ.get("EMERGE_REF_ROOT", "")


class _AnyType:
    def __getitem__(self, item):
        return self

    def __call__(self, *a, **k):
        return self


def _njit(*args, **kwargs):
    if len(args) == 1 and callable(args[0]) and not isinstance(args[0], _AnyType) and not kwargs:
        return args[0]
    return lambda f: f


def _install_numba():
    nb = types.ModuleType("numba")
    nb.njit = _njit
    nb.jit = _njit
    nb.prange = range
    anyt = _AnyType()
    nb.typeof = anyt
    for name in ("f8", "f4", "i8", "i4", "c16", "c8", "b1", "boolean", "int64", "float64",
                 "complex128", "void", "uint8", "int32"):
        setattr(nb, name, anyt)
    nb.types = types.SimpleNamespace(Tuple=anyt, UniTuple=anyt, float64=anyt, int64=anyt,
                                     complex128=anyt, Array=anyt, boolean=anyt, void=anyt)
    sys.modules["numba"] = nb
    sys.modules["numba.types"] = nb.types

    npb = types.ModuleType("numba_progress")

    class ProgressBar:
        def __init__(self, *a, **k):
            pass

        def __enter__(self):
            return self

        def __exit__(self, *a):
            return False

        def update(self, n=1):
            pass

    npb.ProgressBar = ProgressBar
    npb.ProgressBarType = anyt
    sys.modules["numba_progress"] = npb
    npp = types.ModuleType("numba_progress.progress")
    npp.ProgressBarType = anyt
    npb.progress = npp
    sys.modules["numba_progress.progress"] = npp


def _install_loguru():
    lg = types.ModuleType("loguru")

    class _Logger:
        def __getattr__(self, name):
            return lambda *a, **k: None

    lg.logger = _Logger()
    sys.modules["loguru"] = lg


class FakeGmsh(types.ModuleType):
    """The subset of the gmsh API that ``Mesh3D`` uses, backed by arrays.

    Node tags are 1-based (as gmsh's), tet element tags start at 1000001,
    triangle element tags at 1, one volume per material tag.
    """

    def __init__(self):
        super().__init__("gmsh")
        self.model = types.SimpleNamespace()
        self.model.mesh = types.SimpleNamespace(get_nodes=self._get_nodes,
                                                get_elements=self._get_elements)
        self.model.getEntities = lambda dim=-1: []
        # outward normals of the boundary faces by tag (set by the fixture that needs them)
        self.face_normals = {}
        self.model.getNormal = lambda tag, uv: np.asarray(self.face_normals[int(tag)], dtype=float)
        self.model.get_boundary = lambda *a, **k: []
        self.model.getBoundary = self.model.get_boundary
        self.initialize = lambda *a, **k: None
        self.finalize = lambda *a, **k: None
        self.set_mesh(np.zeros((3, 0)), np.zeros((4, 0), dtype=np.int64), {}, np.zeros(0, dtype=np.int64))

    def set_mesh(self, nodes, tets, boundary: dict, cell_tag):
        self.nodes = np.asarray(nodes, dtype=np.float64)
        self.tets = np.asarray(tets, dtype=np.int64)
        self.boundary = {int(k): np.asarray(v, dtype=np.int64) for k, v in boundary.items()}
        self.cell_tag = np.asarray(cell_tag, dtype=np.int64)
        self.tet_etags = np.arange(self.tets.shape[1], dtype=np.int64) + 1000001
        tri_blocks = [self.boundary[k] for k in sorted(self.boundary)]
        self.all_tris = np.concatenate(tri_blocks, axis=1) if tri_blocks else np.zeros((3, 0), dtype=np.int64)
        off = 1
        self.tri_etags = {}
        for k in sorted(self.boundary):
            n = self.boundary[k].shape[1]
            self.tri_etags[k] = np.arange(off, off + n, dtype=np.int64)
            off += n

    def _get_nodes(self, *a, **k):
        n = self.nodes.shape[1]
        return np.arange(1, n + 1, dtype=np.uint64), self.nodes.T.ravel().copy(), np.zeros(0)

    def _get_elements(self, dim=-1, tag=-1):
        if dim == 3:
            if tag == -1:
                sel = np.arange(self.tets.shape[1])
            else:
                sel = np.nonzero(self.cell_tag == tag)[0]
            return ([4], [self.tet_etags[sel].astype(np.uint64)],
                    [(self.tets[:, sel].T.ravel() + 1).astype(np.uint64)])
        if dim == 2:
            if tag == -1:
                tris = self.all_tris
                etags = np.concatenate([self.tri_etags[k] for k in sorted(self.tri_etags)]) \
                    if self.tri_etags else np.zeros(0, dtype=np.int64)
            else:
                tris = self.boundary.get(tag, np.zeros((3, 0), dtype=np.int64))
                etags = self.tri_etags.get(tag, np.zeros(0, dtype=np.int64))
            return ([2], [etags.astype(np.uint64)], [(tris.T.ravel() + 1).astype(np.uint64)])
        raise NotImplementedError(dim)


def install() -> FakeGmsh:
    """Register every stand-in and the ``fem`` namespace packages; return the fake gmsh."""
    if not REF_ROOT or not os.path.isdir(os.path.join(REF_ROOT, "fem")):
        raise RuntimeError("the EMerge checkout is not set: pass --ref PATH to make_golden.py "
                           "or set EMERGE_REF_ROOT to the directory that holds fem/")
    _install_numba()
    _install_loguru()
    g = FakeGmsh()
    sys.modules["gmsh"] = g
    sys.modules["pypardiso"] = types.ModuleType("pypardiso")
    sys.modules["pypardiso"].spsolve = None
    for name, path in (("fem", f"{REF_ROOT}/fem"),
                       ("fem.physics", f"{REF_ROOT}/fem/physics"),
                       ("fem.physics.edm", f"{REF_ROOT}/fem/physics/edm"),
                       ("fem.plotting", f"{REF_ROOT}/fem/plotting"),
                       ("fem.modeling", f"{REF_ROOT}/fem/modeling")):
        m = types.ModuleType(name)
        m.__path__ = [path]
        sys.modules[name] = m
    return g
