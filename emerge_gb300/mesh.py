"""Structured tetrahedral meshes and their edge/face topology.

EMerge builds meshes with gmsh and derives the edge/face topology in
``Mesh3D.update`` (fem/mesh3d.py:224-355).  gmsh is not part of this package,
so this module provides the two pieces the frequency-domain hot path needs:

* ``structured_box`` — an axis-aligned block of hexahedra, each split into six
  Kuhn tetrahedra (all six share the hex's main diagonal, which makes the split
  conforming across neighbouring hexes), with optional interior-vertex jitter
  and per-face boundary-triangle tags.
* ``TetMesh`` — the topology arrays with the same meaning and slot conventions
  as ``Mesh3D``:

  - ``edges (2, nE)``: vertex pairs sorted ascending (fem/mesh3d.py:254-262)
  - ``tris (3, nTri)``: vertex triples sorted ascending (fem/mesh3d.py:263-271)
  - ``tet_to_edge (6, nT)``: local vertex pairs (0,1),(0,2),(0,3),(1,2),(3,1),(2,3)
    (fem/mesh3d.py:290-292)
  - ``tet_to_tri (4, nT)``: local triples (0,1,2),(0,2,3),(0,3,1),(1,2,3)
    (fem/mesh3d.py:296)
  - ``tri_to_edge (3, nTri)``: edges (v0,v1),(v1,v2),(v0,v2) of the sorted
    triple (fem/mesh3d.py:331-335)
  - ``edge_lengths (nE,)`` computed as ``sqrt(sum(d**2))`` (fem/mesh3d.py:351)

The reference numbers edges and faces in CPython ``set`` iteration order; this
module numbers them in ascending (lexicographic) vertex-tuple order instead.
Any numbering is a valid mesh: the assembled matrices are the same operator up
to a symmetric permutation, and the GPU assembler consumes whatever numbering
it is handed (it never renumbers).
"""
from __future__ import annotations

import numpy as np

# Local vertex pairs / triples of the tet edge and face slots (fem/mesh3d.py:290-296).
TET_EDGE_SLOTS = np.array([[0, 0, 0, 1, 3, 2], [1, 2, 3, 2, 1, 3]], dtype=np.int64)
TET_FACE_SLOTS = np.array([[0, 0, 0, 1], [1, 2, 3, 2], [2, 3, 1, 3]], dtype=np.int64)

# Face tags of ``structured_box``: one per side of the box.
FACE_XMIN, FACE_XMAX, FACE_YMIN, FACE_YMAX, FACE_ZMIN, FACE_ZMAX = 1, 2, 3, 4, 5, 6


def _pack(cols: list[np.ndarray], base: int) -> np.ndarray:
    key = np.zeros(cols[0].shape, dtype=np.int64)
    for c in cols:
        key = key * base + c
    return key


class TetMesh:
    """Topology of a tetrahedral mesh (the fields of ``Mesh3D`` the FEM path reads).

    Args:
        nodes: (3, nN) float64 vertex coordinates.
        tets: (4, nT) int64 vertex indices per tetrahedron.
        boundary: optional {face_tag: (3, n) int64 triangle vertex indices}.
        cell_tag: optional (nT,) int64 tag per tet (material/volume id).
        device: build the topology on this CUDA device (``topology.build_topology``)
            instead of with NumPy on the host; the arrays are the same.
    """

    def __init__(self, nodes: np.ndarray, tets: np.ndarray,
                 boundary: dict[int, np.ndarray] | None = None,
                 cell_tag: np.ndarray | None = None, device=None):
        self.nodes = np.ascontiguousarray(nodes, dtype=np.float64)
        self.tets = np.ascontiguousarray(tets, dtype=np.int64)
        self.boundary = {} if boundary is None else {int(k): np.asarray(v, dtype=np.int64)
                                                      for k, v in boundary.items()}
        nT = self.tets.shape[1]
        self.cell_tag = np.zeros(nT, dtype=np.int64) if cell_tag is None else np.asarray(cell_tag, dtype=np.int64)
        if device is None:
            self._build()
        else:
            self._build_device(device)

    # -- sizes (Mesh3D properties, fem/mesh3d.py:118-136)
    @property
    def n_nodes(self) -> int:
        return self.nodes.shape[1]

    @property
    def n_tets(self) -> int:
        return self.tets.shape[1]

    @property
    def n_edges(self) -> int:
        return self.edges.shape[1]

    @property
    def n_tris(self) -> int:
        return self.tris.shape[1]

    def _build(self) -> None:
        nN = self.n_nodes
        T = self.tets
        nT = T.shape[1]
        if nN >= (1 << 21):
            raise ValueError("TetMesh supports up to 2**21 vertices (int64 face keys)")

        # edges: ascending vertex pairs, numbered in ascending key order
        a = T[TET_EDGE_SLOTS[0]]
        b = T[TET_EDGE_SLOTS[1]]
        lo = np.minimum(a, b)
        hi = np.maximum(a, b)
        ekey = _pack([lo, hi], nN)                                 # (6, nT)
        uek, einv = np.unique(ekey.ravel(), return_inverse=True)
        self.edges = np.stack([uek // nN, uek % nN]).astype(np.int64)
        self.tet_to_edge = einv.reshape(6, nT).astype(np.int64)

        # faces: ascending vertex triples
        f = np.sort(np.stack([T[TET_FACE_SLOTS[0]], T[TET_FACE_SLOTS[1]], T[TET_FACE_SLOTS[2]]]), axis=0)
        fkey = _pack([f[0], f[1], f[2]], nN)                       # (4, nT)
        ufk, finv = np.unique(fkey.ravel(), return_inverse=True)
        self.tris = np.stack([ufk // (nN * nN), (ufk // nN) % nN, ufk % nN]).astype(np.int64)
        self.tet_to_tri = finv.reshape(4, nT).astype(np.int64)

        # tri -> edge: (v0,v1), (v1,v2), (v0,v2) of the sorted triple
        t0, t1, t2 = self.tris
        self.tri_to_edge = np.stack([
            np.searchsorted(uek, _pack([t0, t1], nN)),
            np.searchsorted(uek, _pack([t1, t2], nN)),
            np.searchsorted(uek, _pack([t0, t2], nN)),
        ]).astype(np.int64)

        # tri -> tet (first two incident tets, -1 when on the boundary), ascending tet id
        flat = self.tet_to_tri.T.ravel()                          # tet-major order
        tet_of = np.repeat(np.arange(nT, dtype=np.int64), 4)
        order = np.argsort(flat, kind="stable")
        fs = flat[order]
        ts = tet_of[order]
        first = np.searchsorted(fs, np.arange(self.n_tris))
        cnt = np.bincount(fs, minlength=self.n_tris)
        self.tri_to_tet = -np.ones((2, self.n_tris), dtype=np.int64)
        self.tri_to_tet[0] = ts[first]
        two = cnt > 1
        self.tri_to_tet[1, two] = ts[first[two] + 1]

        d = self.nodes[:, self.edges[0]] - self.nodes[:, self.edges[1]]
        self.edge_lengths = np.sqrt(np.sum(d ** 2, axis=0))
        self.centers = self.nodes[:, T].mean(axis=1)
        self._ufk = ufk

    def _build_device(self, device) -> None:
        from .topology import build_topology
        t = build_topology(self.nodes, self.tets, device)
        self.edges, self.tris = t["edges"], t["tris"]
        self.tet_to_edge, self.tet_to_tri = t["tet_to_edge"], t["tet_to_tri"]
        self.tri_to_edge, self.tri_to_tet = t["tri_to_edge"], t["tri_to_tet"]
        self.edge_lengths = t["edge_lengths"]
        self.tet_to_field = t["tet_to_field"]
        self.centers = self.nodes[:, self.tets].mean(axis=1)
        nN = self.n_nodes
        self._ufk = (self.tris[0] * nN + self.tris[1]) * nN + self.tris[2] if nN < (1 << 21) else None

    def get_edge(self, i1: int, i2: int) -> int:
        lo, hi = min(i1, i2), max(i1, i2)
        k = lo * self.n_nodes + hi
        e = int(np.searchsorted(self.edges[0] * self.n_nodes + self.edges[1], k))
        return e

    def tri_ids(self, tri_vertices: np.ndarray) -> np.ndarray:
        """Indices of the faces with the given (3, n) vertex triples (any order)."""
        if self._ufk is None:
            raise ValueError("face lookup by vertex triple supports up to 2**21 vertices")
        s = np.sort(np.asarray(tri_vertices, dtype=np.int64), axis=0)
        key = _pack([s[0], s[1], s[2]], self.n_nodes)
        idx = np.searchsorted(self._ufk, key)
        if np.any(idx >= len(self._ufk)) or np.any(self._ufk[np.minimum(idx, len(self._ufk) - 1)] != key):
            raise ValueError("triangle not in mesh")
        return idx.astype(np.int64)

    def get_triangles(self, face_tags) -> np.ndarray:
        """Face indices of boundary triangles with the given tag(s) (``Mesh3D.get_triangles``)."""
        if isinstance(face_tags, (int, np.integer)):
            face_tags = [int(face_tags)]
        out = [self.tri_ids(self.boundary[t]) for t in face_tags if t in self.boundary]
        return np.concatenate(out) if out else np.zeros(0, dtype=np.int64)


class Nedelec2Basis:
    """Second-order Nédélec DOF numbering (fem/elements/nedelec2.py:32-62).

    DOF blocks: [edge mode 1 | face mode 1 | edge mode 2 | face mode 2], i.e.
    ``n_field = 2*nE + 2*nTri``; ``tet_to_field`` rows 0-5 edge m1, 6-9 face m1,
    10-15 edge m2, 16-19 face m2.
    """

    n_tet_dofs = 20
    n_tri_dofs = 8

    def __init__(self, mesh: TetMesh):
        self.mesh = mesh
        nE, nF = mesh.n_edges, mesh.n_tris
        self.n_edges, self.n_tris, self.n_tets = nE, nF, mesh.n_tets
        self.nedges, self.ntris, self.ntets = nE, nF, mesh.n_tets
        self.n_field = self.nfield = 2 * nE + 2 * nF
        t2f = np.zeros((20, mesh.n_tets), dtype=np.int64)
        t2f[:6] = mesh.tet_to_edge
        t2f[6:10] = mesh.tet_to_tri + nE
        t2f[10:16] = mesh.tet_to_edge + (nF + nE)
        t2f[16:20] = mesh.tet_to_tri + (nF + 2 * nE)
        self.tet_to_field = t2f
        self.edge_to_field = np.stack([np.arange(nE), np.arange(nE) + nF + nE]).astype(np.int64)
        tri2f = np.zeros((8, nF), dtype=np.int64)
        tri2f[:3] = mesh.tri_to_edge
        tri2f[3] = np.arange(nF) + nE
        tri2f[4:7] = mesh.tri_to_edge + nE + nF
        tri2f[7] = np.arange(nF) + 2 * nE + nF
        self.tri_to_field = tri2f


def _axis(n: int, length: float, origin: float = 0.0) -> np.ndarray:
    return origin + np.linspace(0.0, length, n + 1)


def structured_box(xs: np.ndarray, ys: np.ndarray, zs: np.ndarray,
                   jitter: float = 0.0, seed: int = 0,
                   cell_tag_fn=None) -> TetMesh:
    """Kuhn-split tetrahedral mesh of the rectilinear grid ``xs × ys × zs``.

    Args:
        xs, ys, zs: strictly increasing grid lines along each axis.
        jitter: interior vertices move by U[-jitter, +jitter]·h_local per
            coordinate (h_local = the smaller neighbouring spacing on that axis),
            drawn from ``numpy.random.default_rng(seed)``.
        cell_tag_fn: optional f(cx, cy, cz) -> int tag per hex (evaluated at hex
            centres before jitter); all six tets of a hex share the tag.

    Tet ``p * n_hex + h`` is Kuhn simplex ``p`` of hex ``h``.

    Node index = i + (nx+1)*(j + (ny+1)*k).  Boundary tags FACE_XMIN..FACE_ZMAX.
    """
    xs, ys, zs = (np.asarray(v, dtype=np.float64) for v in (xs, ys, zs))
    nx, ny, nz = len(xs) - 1, len(ys) - 1, len(zs) - 1
    X, Y, Z = np.meshgrid(xs, ys, zs, indexing="ij")               # (nx+1, ny+1, nz+1)
    nodes = np.stack([X.transpose(2, 1, 0).ravel(), Y.transpose(2, 1, 0).ravel(),
                      Z.transpose(2, 1, 0).ravel()])
    if jitter > 0:
        rng = np.random.default_rng(seed)
        d = rng.uniform(-jitter, jitter, size=nodes.shape)
        n_id = np.arange(nodes.shape[1])
        grid_idx = (n_id % (nx + 1), (n_id // (nx + 1)) % (ny + 1), n_id // ((nx + 1) * (ny + 1)))
        interior = np.ones(nodes.shape[1], dtype=bool)
        for idx, n in zip(grid_idx, (nx, ny, nz)):
            interior &= (idx > 0) & (idx < n)
        for ax, (g, idx) in enumerate(zip((xs, ys, zs), grid_idx)):
            h = np.diff(g)
            hl = np.minimum(np.r_[h[0], h], np.r_[h, h[-1]])        # per grid line
            nodes[ax] += np.where(interior, d[ax] * hl[idx], 0.0)

    def nid(i, j, k):
        return i + (nx + 1) * (j + (ny + 1) * k)

    I, J, K = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    I, J, K = (v.transpose(2, 1, 0).ravel() for v in (I, J, K))   # hex index = i + nx*(j + ny*k)
    v000 = nid(I, J, K)
    unit = {"x": (1, 0, 0), "y": (0, 1, 0), "z": (0, 0, 1)}
    perms = (("x", "y", "z"), ("x", "z", "y"), ("y", "x", "z"),
             ("y", "z", "x"), ("z", "x", "y"), ("z", "y", "x"))
    tets = []
    for p in perms:
        a = unit[p[0]]
        ab = tuple(u + v for u, v in zip(a, unit[p[1]]))
        tets.append(np.stack([v000, nid(I + a[0], J + a[1], K + a[2]),
                              nid(I + ab[0], J + ab[1], K + ab[2]), nid(I + 1, J + 1, K + 1)]))
    tets = np.stack(tets, axis=1).reshape(4, -1)                   # tet p * n_hex + hex (permutation-major)
    # positive orientation (as gmsh emits): EMerge's field interpolation evaluates the
    # barycentrics with |V| (fem/mth/tet.py:371-497) and so assumes det > 0
    p = nodes[:, tets]                                             # (3, 4, nT)
    d1, d2, d3 = p[:, 1] - p[:, 0], p[:, 2] - p[:, 0], p[:, 3] - p[:, 0]
    neg = np.einsum("it,it->t", d1, np.cross(d2, d3, axis=0)) < 0
    tets[2, neg], tets[3, neg] = tets[3, neg], tets[2, neg].copy()
    if cell_tag_fn is not None:
        cx = 0.5 * (xs[I] + xs[I + 1])
        cy = 0.5 * (ys[J] + ys[J + 1])
        cz = 0.5 * (zs[K] + zs[K + 1])
        cell_tag = np.tile(np.asarray(cell_tag_fn(cx, cy, cz), dtype=np.int64), 6)   # same layout as tets
    else:
        cell_tag = None

    boundary = {}
    # each boundary quad splits along the diagonal the Kuhn tets induce (v000-v111 projection)
    def quads(fixed_axis, fixed_idx, tag):
        ranges = [np.arange(nx), np.arange(ny), np.arange(nz)]
        ranges[fixed_axis] = np.array([fixed_idx])
        A, B, C = np.meshgrid(*ranges, indexing="ij")
        A, B, C = A.ravel(), B.ravel(), C.ravel()
        o = [A, B, C]
        u_ax, v_ax = [ax for ax in range(3) if ax != fixed_axis]
        def shift(du, dv):
            s = [o[0].copy(), o[1].copy(), o[2].copy()]
            s[u_ax] = s[u_ax] + du
            s[v_ax] = s[v_ax] + dv
            return nid(*s)
        p00, p10, p01, p11 = shift(0, 0), shift(1, 0), shift(0, 1), shift(1, 1)
        t1 = np.stack([p00, p10, p11])
        t2 = np.stack([p00, p01, p11])
        boundary[tag] = np.concatenate([t1, t2], axis=1)
    quads(0, 0, FACE_XMIN); quads(0, nx, FACE_XMAX)
    quads(1, 0, FACE_YMIN); quads(1, ny, FACE_YMAX)
    quads(2, 0, FACE_ZMIN); quads(2, nz, FACE_ZMAX)
    return TetMesh(nodes, tets, boundary, cell_tag)


def unit_cube(n: int, jitter: float = 0.0, seed: int = 0) -> TetMesh:
    """Unit cube split into n³ hexes × 6 Kuhn tets (the assembly micro-benchmark mesh)."""
    g = _axis(n, 1.0)
    return structured_box(g, g, g, jitter=jitter, seed=seed)
