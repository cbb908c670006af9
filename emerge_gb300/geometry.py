"""Benchmark geometries of the frequency-domain path, meshed with structured Kuhn tets.

gmsh is not available, so the structures are built on rectilinear grids whose
lines are snapped to every material / metal face, with metal regions removed
and their surfaces made PEC.  All lengths in metres.

* ``straight_waveguide`` — WR-90-like guide 22.86 x 10.16 x 50 mm, PEC walls,
  TE10 waveports on both ends (the reference's boundary_selection_test.py setup).
* ``iris_filter`` — five-cavity WR-90 bandpass filter: six inductive irises
  2 mm thick with centred apertures [12.0, 8.5, 7.8, 7.8, 8.5, 12.0] mm, cavity
  lengths [15.8, 17.6, 18.0, 17.6, 15.8] mm, 10 mm feed guides.
* ``patch_antenna`` — rectangular patch on a lossy substrate over a finite ground
  plane, fed by a lumped port between ground and patch, in an air box closed by
  first-order absorbing walls (the patch benchmark's layout at a coarser grid).
* ``dielectric_cavity`` — PEC box with a centred full-height dielectric cylinder
  (staircased on the grid), the eigenmode workload; ``cavity_set`` draws a batch
  of them from a seed.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .bc import PEC, AbsorbingBoundary, CoordinateSystem, LumpedPort, RectangularWaveguide
from .mesh import FACE_XMAX, FACE_XMIN, FACE_YMAX, FACE_YMIN, FACE_ZMAX, FACE_ZMIN, Nedelec2Basis, TetMesh, structured_box

TAG_PORT1, TAG_PORT2, TAG_PEC = 11, 12, 13


@dataclass
class Problem:
    mesh: TetMesh
    field: Nedelec2Basis
    bcs: list
    er: np.ndarray
    ur: np.ndarray
    name: str


def _lines(breaks, h):
    """Grid lines through every break point, spacing at most h in between."""
    out = [breaks[0]]
    for a, b in zip(breaks[:-1], breaks[1:]):
        n = max(1, int(np.ceil((b - a) / h - 1e-9)))
        out.extend(list(a + (b - a) * np.arange(1, n + 1) / n))
    return np.array(out)


def _classify_boundary(mesh: TetMesh, L: float) -> dict:
    bnd = np.flatnonzero(mesh.tri_to_tet[1] < 0)
    tv = mesh.tris[:, bnd]
    y = mesh.nodes[1][tv]
    tol = 1e-9
    p1 = np.all(np.abs(y) < tol, axis=0)
    p2 = np.all(np.abs(y - L) < tol, axis=0)
    return {TAG_PORT1: tv[:, p1], TAG_PORT2: tv[:, p2], TAG_PEC: tv[:, ~(p1 | p2)]}


def _guide_problem(xs, ys, zs, metal_fn, a, b, L, name):
    box = structured_box(xs, ys, zs, cell_tag_fn=metal_fn)
    keep = box.cell_tag == 0
    mesh = TetMesh(box.nodes, box.tets[:, keep])
    mesh = TetMesh(mesh.nodes, mesh.tets, boundary=_classify_boundary(mesh, L))
    field = Nedelec2Basis(mesh)
    p1 = RectangularWaveguide([TAG_PORT1], 1, CoordinateSystem([1.0, 0, 0], [0, 0, 1.0], [0, -1.0, 0],
                                                               [a / 2, 0.0, b / 2]), (a, b))
    p2 = RectangularWaveguide([TAG_PORT2], 2, CoordinateSystem([-1.0, 0, 0], [0, 0, 1.0], [0, 1.0, 0],
                                                               [a / 2, L, b / 2]), (a, b))
    nT = mesh.n_tets
    eye = np.repeat(np.eye(3, dtype=np.complex128)[:, :, None], nT, axis=2)
    return Problem(mesh, field, [PEC([TAG_PEC]), p1, p2], eye, eye.copy(), name)


def straight_waveguide(h: float = 3e-3, a: float = 0.02286, b: float = 0.01016, L: float = 0.05) -> Problem:
    xs = _lines([0.0, a], h)
    ys = _lines([0.0, L], h)
    zs = _lines([0.0, b], h)
    return _guide_problem(xs, ys, zs, lambda cx, cy, cz: np.zeros_like(cx, dtype=np.int64), a, b, L,
                          f"WR-90 straight guide, h={h * 1e3:.2f} mm")


IRIS_APERTURES = [12.0e-3, 8.5e-3, 7.8e-3, 7.8e-3, 8.5e-3, 12.0e-3]
CAVITIES = [15.8e-3, 17.6e-3, 18.0e-3, 17.6e-3, 15.8e-3]


def iris_filter(h: float = 2e-3, a: float = 0.02286, b: float = 0.01016, t: float = 2e-3,
                feed: float = 10e-3, hy: float | None = None) -> Problem:
    """The five-cavity filter with grid spacing at most ``h`` across the guide and ``hy``
    (default ``h``) along it.  Every element stays within the maximum element size
    ``h``; a smaller ``hy`` adds cross-sections, which is how the structured grid reaches
    the DOF count of a free mesh of the same maximum size (h = 2 mm, hy = 1.3 mm: about
    3·10^5 DOFs)."""
    hy = h if hy is None else hy
    # y positions of the iris slabs
    y = feed
    slabs = []
    for i, w in enumerate(IRIS_APERTURES):
        slabs.append((y, y + t, w))
        y += t
        if i < len(CAVITIES):
            y += CAVITIES[i]
    L = y + feed
    ybreaks = sorted({0.0, L} | {s[0] for s in slabs} | {s[1] for s in slabs})
    xbreaks = sorted({0.0, a} | {(a - w) / 2 for w in IRIS_APERTURES} | {(a + w) / 2 for w in IRIS_APERTURES})
    xs = _lines(xbreaks, h)
    ys = _lines(ybreaks, hy)
    zs = _lines([0.0, b], h)

    def metal(cx, cy, cz):
        m = np.zeros_like(cx, dtype=bool)
        for y0, y1, w in slabs:
            in_slab = (cy > y0) & (cy < y1)
            outside = (cx < (a - w) / 2) | (cx > (a + w) / 2)
            m |= in_slab & outside
        return m.astype(np.int64)

    name = f"5-cavity WR-90 iris filter, h={h * 1e3:.2f} mm" + (f", hy={hy * 1e3:.2f} mm" if hy != h else "")
    return _guide_problem(xs, ys, zs, metal, a, b, L, name)


TAG_GROUND, TAG_PATCH, TAG_FEED = 21, 22, 23


def _plane_tris(mesh: TetMesh, axis: int, value: float, lo, hi) -> np.ndarray:
    """(3, n) vertex triples of the mesh faces in the plane x_axis = value whose other two
    coordinates lie in [lo, hi] (per axis, ascending axis order)."""
    P = mesh.nodes[:, mesh.tris]                                   # (3, 3, nTri)
    tol = 1e-9
    on = np.all(np.abs(P[axis] - value) < tol, axis=0)
    for k, a in enumerate([a for a in range(3) if a != axis]):
        on &= np.all((P[a] >= lo[k] - tol) & (P[a] <= hi[k] + tol), axis=0)
    return mesh.tris[:, on]


def patch_antenna(h_air: float = 12.5e-3, h_patch: float = 5e-3, L: float = 40e-3, W: float = 30e-3,
                  t: float = 1.52e-3, ground: float = 80e-3, margin: float = 37.5e-3, eps_r: float = 3.38,
                  tand: float = 0.0027, feed_x: float = -10e-3, feed_w: float = 5e-3, Z0: float = 50.0) -> Problem:
    """Patch antenna: an L x W PEC patch at z = t on a t-thick substrate (eps_r (1 - j tand)),
    over a ground x ground PEC plane at z = 0, in an air box ``margin`` beyond the ground
    on every side (below included) with first-order absorbing walls.  A lumped port
    (``Z0``, E along +z) fills the ``feed_w`` x t rectangle at x = feed_x, centred in y,
    between ground and patch.  The grid is snapped to every edge; spacing at most
    h_patch over the ground plane, h_air outside, one cell across the substrate."""
    g, B = ground / 2, ground / 2 + margin
    xb = sorted({-B, -g, -L / 2, feed_x, L / 2, g, B})
    yb = sorted({-B, -g, -W / 2, -feed_w / 2, feed_w / 2, W / 2, g, B})

    def lines(breaks):
        out = [breaks[0]]
        for a, b in zip(breaks[:-1], breaks[1:]):
            h = h_patch if (a >= -g - 1e-12 and b <= g + 1e-12) else h_air
            n = max(1, int(np.ceil((b - a) / h - 1e-9)))
            out.extend(list(a + (b - a) * np.arange(1, n + 1) / n))
        return np.array(out)

    xs, ys = lines(xb), lines(yb)
    zs = np.concatenate([_lines([-margin, 0.0], h_air), [t], _lines([t, t + margin], h_air)[1:]])

    def substrate(cx, cy, cz):
        return ((np.abs(cx) < g) & (np.abs(cy) < g) & (cz > 0) & (cz < t)).astype(np.int64)

    box = structured_box(xs, ys, zs, cell_tag_fn=substrate)
    bnd = dict(box.boundary)
    bnd[TAG_GROUND] = _plane_tris(box, 2, 0.0, (-g, -g), (g, g))
    bnd[TAG_PATCH] = _plane_tris(box, 2, t, (-L / 2, -W / 2), (L / 2, W / 2))
    bnd[TAG_FEED] = _plane_tris(box, 0, feed_x, (-feed_w / 2, 0.0), (feed_w / 2, t))
    mesh = TetMesh(box.nodes, box.tets, boundary=bnd, cell_tag=box.cell_tag)
    field = Nedelec2Basis(mesh)
    nT = mesh.n_tets
    er = np.repeat(np.eye(3, dtype=np.complex128)[:, :, None], nT, axis=2)
    er[[0, 1, 2], [0, 1, 2], :] = np.where(mesh.cell_tag == 1, eps_r * (1 - 1j * tand), 1.0)[None, :]
    ur = np.repeat(np.eye(3, dtype=np.complex128)[:, :, None], nT, axis=2)
    feed = LumpedPort([TAG_FEED], 1, width=feed_w, height=t, direction=(0, 0, 1), normal=(1, 0, 0), Z0=Z0)
    bcs = [PEC([TAG_GROUND, TAG_PATCH]),
           AbsorbingBoundary([FACE_XMIN, FACE_XMAX, FACE_YMIN, FACE_YMAX, FACE_ZMIN, FACE_ZMAX]), feed]
    return Problem(mesh, field, bcs, er, ur,
                   f"patch {L * 1e3:.0f}x{W * 1e3:.0f} mm on {t * 1e3:.2f} mm eps_r={eps_r}, ground "
                   f"{ground * 1e3:.0f} mm, air margin {margin * 1e3:.1f} mm, h={h_patch * 1e3:.1f}/{h_air * 1e3:.1f} mm")


def dielectric_cavity(a: float, b: float, c: float, radius: float, eps_r: float, h: float) -> Problem:
    """PEC box a x b x c with a centred cylinder (axis z, full height) of permittivity eps_r.

    Cells whose centre lies inside the cylinder carry eps_r (a staircased cylinder);
    the grid spacing is at most h.  All six faces are PEC; no ports."""
    xs = _lines([0.0, a], h)
    ys = _lines([0.0, b], h)
    zs = _lines([0.0, c], h)

    def inside(cx, cy, cz):
        return (((cx - a / 2) ** 2 + (cy - b / 2) ** 2) < radius ** 2).astype(np.int64)

    mesh = structured_box(xs, ys, zs, cell_tag_fn=inside)
    field = Nedelec2Basis(mesh)
    nT = mesh.n_tets
    er = np.repeat(np.eye(3, dtype=np.complex128)[:, :, None], nT, axis=2)
    er[[0, 1, 2], [0, 1, 2], :] = np.where(mesh.cell_tag == 1, eps_r, 1.0)[None, :]
    ur = np.repeat(np.eye(3, dtype=np.complex128)[:, :, None], nT, axis=2)
    pec = PEC([FACE_XMIN, FACE_XMAX, FACE_YMIN, FACE_YMAX, FACE_ZMIN, FACE_ZMAX])
    return Problem(mesh, field, [pec], er, ur,
                   f"PEC cavity {a * 1e3:.1f}x{b * 1e3:.1f}x{c * 1e3:.1f} mm, cylinder r={radius * 1e3:.2f} mm "
                   f"eps={eps_r:.2f}, h={h * 1e3:.2f} mm")


def cavity_set(n: int = 64, seed: int = 4, h: float = 2e-3):
    """Seeded batch of dielectric cavities: sides ~ U[15, 40] mm, radius ~ U[2, 6] mm,
    eps_r ~ U[2, 30] (numpy default_rng(seed)).  Returns a list of Problems."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        a, b, c = rng.uniform(15e-3, 40e-3, 3)
        r = min(rng.uniform(2e-3, 6e-3), 0.45 * min(a, b))
        eps = rng.uniform(2.0, 30.0)
        out.append(dielectric_cavity(a, b, c, r, eps, h))
    return out
