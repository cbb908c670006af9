"""GPU mesh topology (emg_topology_create) against the host builder of mesh.py.

The arrays are integer and index work: they must be bitwise equal, and the edge
lengths bitwise equal to NumPy's sqrt(sum(d**2)).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from emerge_gb300 import _build
    _build.build()
    return torch


def _assert_same(host, dev):
    from emerge_gb300.mesh import Nedelec2Basis
    for name in ("edges", "tris", "tet_to_edge", "tet_to_tri", "tri_to_edge", "tri_to_tet"):
        assert np.array_equal(getattr(host, name), getattr(dev, name)), name
    assert np.array_equal(host.edge_lengths.view(np.int64), dev.edge_lengths.view(np.int64))
    assert np.array_equal(Nedelec2Basis(host).tet_to_field, dev.tet_to_field)
    assert np.array_equal(host.centers, dev.centers)


@pytest.mark.parametrize("n", [1, 5, 12])
def test_cube_topology_matches_host(cuda, n):
    from emerge_gb300.mesh import TetMesh, unit_cube
    m = unit_cube(n, jitter=0.15, seed=n)
    d = TetMesh(m.nodes, m.tets, device="cuda")
    _assert_same(m, d)


def test_shuffled_tets_and_vertex_order(cuda):
    """Tet order, vertex labels and the vertex order inside each tet are arbitrary."""
    from emerge_gb300.mesh import TetMesh, unit_cube
    rng = np.random.default_rng(3)
    m = unit_cube(6, jitter=0.1, seed=2)
    relabel = rng.permutation(m.n_nodes)
    nodes = np.empty_like(m.nodes)
    nodes[:, relabel] = m.nodes
    tets = relabel[m.tets][:, rng.permutation(m.n_tets)]
    for t in range(tets.shape[1]):
        tets[:, t] = tets[rng.permutation(4), t]
    host = TetMesh(nodes, tets)
    dev = TetMesh(nodes, tets, device="cuda")
    _assert_same(host, dev)


def test_iris_filter_topology_matches_host(cuda):
    from emerge_gb300.geometry import iris_filter
    from emerge_gb300.mesh import TetMesh
    m = iris_filter(4e-3).field.mesh
    dev = TetMesh(m.nodes, m.tets, device="cuda")
    _assert_same(m, dev)


def test_single_tet_and_empty_mesh(cuda):
    from emerge_gb300.mesh import TetMesh
    from emerge_gb300.topology import build_topology
    nodes = np.array([[0, 1, 0, 0], [0, 0, 1, 0], [0, 0, 0, 1]], dtype=float)
    tets = np.array([[0], [1], [2], [3]])
    _assert_same(TetMesh(nodes, tets), TetMesh(nodes, tets, device="cuda"))
    t = build_topology(nodes, np.zeros((4, 0), dtype=np.int64))
    assert t["edges"].shape == (2, 0) and t["tris"].shape == (3, 0) and t["tet_to_field"].shape == (20, 0)


def test_invalid_meshes_are_rejected(cuda):
    from emerge_gb300._lib import EmgError
    from emerge_gb300.topology import build_topology
    nodes = np.zeros((3, 5))
    with pytest.raises(EmgError):                       # vertex index out of range
        build_topology(nodes, np.array([[0], [1], [2], [7]]))
    # three tets on the face (0, 1, 2)
    with pytest.raises(EmgError):
        build_topology(nodes, np.array([[0, 0, 0], [1, 1, 1], [2, 2, 2], [3, 4, 4]]))
