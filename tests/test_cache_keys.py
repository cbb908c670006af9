"""Cache keys of the solver pattern analysis and of the assembly plan (CPU only)."""
import types

import numpy as np
import scipy.sparse as sp


def test_solver_pattern_key_sees_every_column():
    """Two patterns with the same row lengths and the same first 4096 column indices
    (a renumbered mesh of the same structure) must not share a solver cache entry."""
    from emerge_gb300.solver import pattern_key
    rng = np.random.default_rng(0)
    n, per_row = 3000, 4
    cols = np.sort(np.stack([rng.choice(n, per_row, replace=False) for _ in range(n)]), axis=1)
    indptr = np.arange(0, n * per_row + 1, per_row)
    a = sp.csr_matrix((np.ones(n * per_row), cols.ravel(), indptr), shape=(n, n))
    cols2 = cols.copy()
    r = n - 1                                  # last row: far beyond the first 4096 indices
    free = np.setdiff1d(np.arange(n), cols2[r])
    cols2[r, -1] = free[-1]
    cols2[r] = np.sort(cols2[r])
    b = sp.csr_matrix((np.ones(n * per_row), cols2.ravel(), indptr), shape=(n, n))
    assert np.array_equal(a.indptr, b.indptr)
    assert np.array_equal(a.indices[:4096], b.indices[:4096])
    assert pattern_key(a) != pattern_key(b)
    assert pattern_key(a) == pattern_key(a.copy())


def test_assembly_plan_follows_mesh_arrays():
    """The plan cached on a field is reused only while the field holds the same arrays."""
    from emerge_gb300.assembly import AssemblyPlan
    m = types.SimpleNamespace(nodes=np.zeros((3, 4)), tets=np.zeros((4, 1)), edges=np.zeros((2, 6)),
                              tris=np.zeros((3, 4)))
    field = types.SimpleNamespace(mesh=m, tet_to_field=np.zeros((20, 1)))
    plan = object.__new__(AssemblyPlan)
    plan._source = (m.nodes, m.tets, m.edges, m.tris, field.tet_to_field)
    assert plan.matches(field)
    m.nodes = m.nodes + 1.0                    # moved geometry, same tet count
    assert not plan.matches(field)
    m.nodes = plan._source[0]
    field.tet_to_field = field.tet_to_field.copy()
    assert not plan.matches(field)
