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


def test_cell_tags_follow_their_hexes():
    """Every tet carries the tag of the hex it was cut from (tagged by hex centre)."""
    from emerge_gb300.mesh import structured_box
    xs = np.array([0.0, 1.0, 2.0, 3.0])
    ys = np.array([0.0, 0.5, 1.5])
    zs = np.array([0.0, 1.0, 2.0])
    box = structured_box(xs, ys, zs, cell_tag_fn=lambda cx, cy, cz: ((cx > 1.0) & (cx < 2.0) & (cz < 1.0)).astype(int))
    c = box.nodes[:, box.tets].mean(axis=1)
    inside = (c[0] > 1.0) & (c[0] < 2.0) & (c[2] < 1.0)
    assert np.array_equal(box.cell_tag == 1, inside)
    assert box.cell_tag.sum() == 6 * 2    # one x-cell x two y-cells x one z-cell, 6 tets each


def test_iris_filter_keeps_only_apertures_in_iris_slabs():
    from emerge_gb300.geometry import IRIS_APERTURES, iris_filter
    p = iris_filter(3e-3)
    c = p.mesh.nodes[:, p.mesh.tets].mean(axis=1)
    a = 0.02286
    y = 10e-3
    for i, w in enumerate(IRIS_APERTURES):
        sel = (c[1] > y) & (c[1] < y + 2e-3)
        assert sel.any()
        assert np.all(c[0, sel] > (a - w) / 2) and np.all(c[0, sel] < (a + w) / 2)
        y += 2e-3 + ([15.8e-3, 17.6e-3, 18.0e-3, 17.6e-3, 15.8e-3] + [0.0])[i]


def test_locality_key_pairs_entity_dofs():
    """The slab order key is a permutation and puts the two DOFs of every kept edge
    or face next to each other."""
    from emerge_gb300.bc import PEC
    from emerge_gb300.freq import Assembler
    from emerge_gb300.mesh import FACE_XMIN, FACE_ZMAX, Nedelec2Basis, unit_cube
    from emerge_gb300.solver import locality_key
    field = Nedelec2Basis(unit_cube(3, jitter=0.1, seed=2))
    sid = Assembler(device="cpu").solve_ids(field, [PEC([FACE_XMIN, FACE_ZMAX])])
    key = locality_key(field, sid)
    assert np.array_equal(np.sort(key), np.arange(sid.size))
    nE, nF = field.mesh.edges.shape[1], field.mesh.tris.shape[1]
    pos = {int(g): i for i, g in enumerate(sid)}
    for g, i in pos.items():
        if g < nE + nF and g + nE + nF in pos:
            assert key[pos[g + nE + nF]] == key[i] + 1


def test_patch_antenna_geometry():
    """Interior PEC sheets, the feed sheet and the substrate of the patch case."""
    from emerge_gb300.geometry import TAG_FEED, TAG_GROUND, TAG_PATCH, patch_antenna
    p = patch_antenna()
    m = p.mesh
    z = m.nodes[2]
    g = m.nodes[:, m.boundary[TAG_GROUND]]
    assert np.all(np.abs(g[2]) < 1e-12) and np.all(np.abs(g[:2]) <= 0.04 + 1e-12)
    pt = m.nodes[:, m.boundary[TAG_PATCH]]
    assert np.all(np.abs(pt[2] - 1.52e-3) < 1e-12)
    assert np.all(np.abs(pt[0]) <= 0.02 + 1e-12) and np.all(np.abs(pt[1]) <= 0.015 + 1e-12)
    # sheet areas: 80 x 80 mm ground, 40 x 30 mm patch, 5 x 1.52 mm feed
    def area(tags):
        tv = m.boundary[tags]
        a, b, c = m.nodes[:, tv[0]], m.nodes[:, tv[1]], m.nodes[:, tv[2]]
        return 0.5 * np.linalg.norm(np.cross((b - a).T, (c - a).T), axis=1).sum()
    assert abs(area(TAG_GROUND) - 0.08 ** 2) < 1e-12
    assert abs(area(TAG_PATCH) - 0.04 * 0.03) < 1e-12
    assert abs(area(TAG_FEED) - 0.005 * 1.52e-3) < 1e-15
    # the sheets are interior faces (two tets each), the substrate fills the slab under the patch
    for tag in (TAG_GROUND, TAG_PATCH, TAG_FEED):
        ids = m.tri_ids(m.boundary[tag])
        assert np.all(m.tri_to_tet[1, ids] >= 0)
    sub = m.cell_tag == 1
    cz = m.nodes[2][m.tets[:, sub]].mean(axis=0)
    assert np.all((cz > 0) & (cz < 1.52e-3))
    assert np.isclose(p.er[0, 0][sub], 3.38 * (1 - 0.0027j)).all()
    # the feed's voltage line runs from ground to patch through the feed centre
    feed = p.bcs[2]
    mid, step = feed.integration_line(m)
    assert np.allclose(mid[:2].T, [[-0.01, 0.0]] * 10) and np.allclose(step.sum(axis=1), [0, 0, 1.52e-3])
    assert z.min() == -0.0375 and abs(z.max() - (1.52e-3 + 0.0375)) < 1e-12


def test_assembler_caches_follow_objects(monkeypatch):
    """Assembler caches are keyed on the field and material objects themselves."""
    import types
    from emerge_gb300 import freq
    built = []

    class FakePlan:
        def assemble_materials(self, er, ur):
            built.append((er, ur))
            return f"E{len(built)}", f"B{len(built)}"

    monkeypatch.setattr(freq, "plan_for", lambda field, device: FakePlan())
    monkeypatch.setattr(freq, "_RobinPlan", lambda field, plan, tris: ("robin", id(field), len(tris)))
    asm = freq.Assembler(device="cpu")
    f1 = types.SimpleNamespace(mesh=types.SimpleNamespace(get_triangles=lambda tags: np.arange(3)))
    er, ur = np.ones((3, 3, 2)), np.ones((3, 3, 2))
    p, E, B = asm._volume(f1, er, ur)
    assert (E, B) == ("E1", "B1")
    assert asm._volume(f1, er, ur)[1] == "E1" and len(built) == 1          # same objects: cached
    assert asm._volume(f1, er.copy(), ur)[1] == "E2"                       # new material array
    f2 = types.SimpleNamespace(mesh=f1.mesh)
    assert asm._volume(f2, er, ur)[1] == "E3"                              # new field
    bc = types.SimpleNamespace(tags=[1])
    r1 = asm._robin_plan(f1, p, bc)
    assert asm._robin_plan(f1, p, bc) is r1
    assert asm._robin_plan(f2, p, bc) is not r1


def test_sparameters_of_mixed_port_types():
    """FrequencySweep._sparams with a waveport and a lumped port: S_ij = pfield_i / pmode_j
    with each port's own formula (fem/physics/edm/emfreq3d.py:735-766, fem/mth/sparam.py)."""
    import types
    import torch
    from emerge_gb300.solver import FrequencySweep
    rng = np.random.default_rng(4)
    n, nf = 40, 3
    wave = types.SimpleNamespace(port_number=1, Zmode=lambda k0: 376.73)
    lump = types.SimpleNamespace(port_number=2, v_integration=True, integration_line=None, voltage=10.0, Z0=50.0)
    sw = object.__new__(FrequencySweep)
    sw.ports = [wave, lump]
    u = rng.normal(size=(n, 2)) + 1j * rng.normal(size=(n, 2))
    sw.u_r = torch.as_tensor(u)
    sw.u_w = sw.u_r
    sw.Pmode = np.array([2.5, 0.0])
    r = torch.as_tensor(rng.choice(n, 6, replace=False))
    w = torch.as_tensor(rng.normal(size=6) + 0j)
    sw._vfun = {1: (r, w)}
    X = rng.normal(size=(n, nf * 2)) + 1j * rng.normal(size=(n, nf * 2))
    k0 = np.array([100.0, 150.0, 200.0])
    S = sw._sparams(torch.as_tensor(X), nf, np.ones((2, nf)), k0)
    V0, Z0, P = 10.0, 50.0, 2.5
    for f in range(nf):
        for j in range(2):
            c = f * 2 + j
            pm = P / (2 * 376.73) if j == 0 else np.sqrt(V0 ** 2 / (2 * Z0))
            G = -(u[:, 0] @ X[:, c])
            V = np.sum(w.numpy() * X[r.numpy(), c])
            pf = [(G - (P if j == 0 else 0.0)) / (2 * 376.73),
                  np.sqrt((V - (V0 if j == 1 else 0.0)) ** 2 / (2 * Z0))]
            for i in range(2):
                assert np.isclose(S[f, i, j], pf[i] / pm, rtol=1e-12, atol=0)
