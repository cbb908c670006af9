"""Project mesh topology against the reference Mesh3D arrays (CPU).

The reference numbers edges/faces in CPython set order; the project in sorted
order.  The tests compare numbering-independent content: the same edge and
face sets, the same per-tet slot contents, and the same tri->edge triples.
"""
import numpy as np

from _fixtures import load
from emerge_gb300.mesh import Nedelec2Basis, structured_box, unit_cube


def _small_box():
    xs = np.array([0.0, 0.4, 1.0])
    return structured_box(xs, xs * 0.8, xs * 1.3 + 0.5, jitter=0.15, seed=3)


def test_topology_matches_reference_as_sets():
    z = load("small_assembly.npz")
    m = _small_box()
    assert np.array_equal(m.nodes, z["nodes"])
    assert np.array_equal(m.tets, z["tets"])
    ref_edges = {tuple(e) for e in z["edges"].T}
    ref_tris = {tuple(t) for t in z["tris"].T}
    assert {tuple(e) for e in m.edges.T} == ref_edges
    assert {tuple(t) for t in m.tris.T} == ref_tris
    # per-tet slot contents (vertex pairs / triples) agree slot by slot
    for s in range(6):
        assert np.array_equal(m.edges[:, m.tet_to_edge[s]], z["edges"][:, z["tet_to_edge"][s]])
    for s in range(4):
        assert np.array_equal(m.tris[:, m.tet_to_tri[s]], z["tris"][:, z["tet_to_tri"][s]])
    # tri -> edge (v0v1, v1v2, v0v2)
    ref = {tuple(z["tris"][:, i]): tuple(tuple(z["edges"][:, e]) for e in z["tri_to_edge"][:, i])
           for i in range(z["tris"].shape[1])}
    mine = {tuple(m.tris[:, i]): tuple(tuple(m.edges[:, e]) for e in m.tri_to_edge[:, i]) for i in range(m.n_tris)}
    assert mine == ref
    # edge lengths of identical edges are bitwise identical
    rl = {tuple(e): l for e, l in zip(z["edges"].T, z["edge_lengths"])}
    assert all(rl[tuple(e)] == l for e, l in zip(m.edges.T, m.edge_lengths))


def test_tets_positively_oriented():
    m = unit_cube(5, jitter=0.15, seed=0)
    p = m.nodes[:, m.tets]
    d1, d2, d3 = p[:, 1] - p[:, 0], p[:, 2] - p[:, 0], p[:, 3] - p[:, 0]
    assert (np.einsum("it,it->t", d1, np.cross(d2, d3, axis=0)) > 0).all()


def test_kuhn_counts():
    """C0 waveguide mesh: 3264 tets, 4545 edges, 7000 faces, 23090 DOFs."""
    xs = np.linspace(0, 0.02286, 9)
    ys = np.linspace(0, 0.05, 18)
    zs = np.linspace(0, 0.01016, 5)
    m = structured_box(xs, ys, zs)
    b = Nedelec2Basis(m)
    assert (m.n_tets, m.n_edges, m.n_tris, b.n_field) == (3264, 4545, 7000, 23090)
    n = 20
    c = unit_cube(n)
    assert c.n_tets == 6 * n ** 3
    # Euler characteristic of a ball: V - E + F - T = 1
    assert c.n_nodes - c.n_edges + c.n_tris - c.n_tets == 1


def test_boundary_tags_cover_the_surface():
    m = unit_cube(3)
    bnd = m.get_triangles([1, 2, 3, 4, 5, 6])
    assert len(np.unique(bnd)) == len(bnd) == (m.tri_to_tet[1] < 0).sum()
