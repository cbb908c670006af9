"""Benchmark geometries of the frequency-domain path, meshed with structured Kuhn tets.

gmsh is not available, so the structures are built on rectilinear grids whose
lines are snapped to every material / metal face, with metal regions removed
and their surfaces made PEC.  All lengths in metres.

* ``straight_waveguide`` — WR-90-like guide 22.86 x 10.16 x 50 mm, PEC walls,
  TE10 waveports on both ends (the reference's boundary_selection_test.py setup).
* ``iris_filter`` — five-cavity WR-90 bandpass filter: six inductive irises
  2 mm thick with centred apertures [12.0, 8.5, 7.8, 7.8, 8.5, 12.0] mm, cavity
  lengths [15.8, 17.6, 18.0, 17.6, 15.8] mm, 10 mm feed guides.
* ``dielectric_cavity`` — PEC box with a centred full-height dielectric cylinder
  (staircased on the grid), the eigenmode workload; ``cavity_set`` draws a batch
  of them from a seed.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .bc import PEC, CoordinateSystem, RectangularWaveguide
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
                feed: float = 10e-3) -> Problem:
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
    ys = _lines(ybreaks, h)
    zs = _lines([0.0, b], h)

    def metal(cx, cy, cz):
        m = np.zeros_like(cx, dtype=bool)
        for y0, y1, w in slabs:
            in_slab = (cy > y0) & (cy < y1)
            outside = (cx < (a - w) / 2) | (cx > (a + w) / 2)
            m |= in_slab & outside
        return m.astype(np.int64)

    return _guide_problem(xs, ys, zs, metal, a, b, L, f"5-cavity WR-90 iris filter, h={h * 1e3:.2f} mm")


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
