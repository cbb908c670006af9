"""CUDA assembly path (through the C ABI) against the reference fixtures and the oracle.

Tolerance: values within 1e-12 of the largest |value| of their CSR row; the
pattern (indptr, indices) bit-exact.
"""
import numpy as np
import pytest

import oracle
from _fixtures import csr_from, field_from, load, rel_to_rowmax

pytestmark = pytest.mark.gpu

TOL = 1e-12


@pytest.fixture(scope="module")
def torch_cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from emerge_gb300 import _build
    _build.build()
    return torch


def _random_materials(nT, seed, mu_one=True):
    rng = np.random.default_rng(seed)
    er = (rng.uniform(1, 10, nT) * (1 - 1j * rng.uniform(0.001, 0.02, nT)))
    ur = np.ones(nT, dtype=np.complex128) if mu_one else rng.uniform(0.5, 3, nT) + 0j
    eye = np.eye(3)[:, :, None]
    return eye * er[None, None, :], eye * ur[None, None, :]


@pytest.mark.parametrize("tag", ["a", "b"])
def test_small_assembly_matches_reference(torch_cuda, tag):
    from emerge_gb300.assembly import tet_mass_stiffness_matrices
    z = load("small_assembly.npz")
    field = field_from(z)
    E, B = tet_mass_stiffness_matrices(field, z["er_" + tag], z["ur_" + tag])
    assert rel_to_rowmax(E, csr_from(z, "E_" + tag)) <= TOL
    assert rel_to_rowmax(B, csr_from(z, "B_" + tag)) <= TOL


def test_waveguide_checksums_match_reference(torch_cuda):
    from emerge_gb300.assembly import tet_mass_stiffness_matrices
    z = load("waveguide.npz")
    field = field_from(z)
    nT = field.mesh.n_tets
    eye = np.repeat(np.eye(3, dtype=np.complex128)[:, :, None], nT, axis=2)
    E, B = tet_mass_stiffness_matrices(field, eye, eye)
    n = E.shape[0]
    w = (np.arange(n) + 1.0) / n
    for name, M in (("E", E), ("B", B)):
        assert M.nnz == int(z[name + "_nnz"])
        assert np.array_equal(M.indptr, z[name + "_indptr"])
        scale = np.abs(M).max(axis=1).toarray().ravel()
        assert np.max(np.abs(np.asarray(M.sum(axis=1)).ravel() - z[name + "_rowsum"]) / scale) <= TOL
        assert np.max(np.abs(M @ w - z[name + "_rowmom"]) / scale) <= TOL


@pytest.mark.parametrize("n,mu_one", [(6, True), (11, False)])
def test_jittered_cube_matches_oracle(torch_cuda, n, mu_one):
    from emerge_gb300.assembly import tet_mass_stiffness_matrices
    from emerge_gb300.mesh import Nedelec2Basis, unit_cube
    m = unit_cube(n, jitter=0.15, seed=n)
    field = Nedelec2Basis(m)
    er, ur = _random_materials(m.n_tets, n, mu_one)
    E, B = tet_mass_stiffness_matrices(field, er, ur)
    Eo, Bo = oracle.tet_mass_stiffness_matrices(field, er, ur)
    assert rel_to_rowmax(E, Eo) <= TOL
    assert rel_to_rowmax(B, Bo) <= TOL


def test_device_path_is_deterministic(torch_cuda):
    torch = torch_cuda
    from emerge_gb300.assembly import AssemblyPlan, material_scalars
    from emerge_gb300.mesh import Nedelec2Basis, unit_cube
    m = unit_cube(9, jitter=0.15, seed=1)
    field = Nedelec2Basis(m)
    er, ur = _random_materials(m.n_tets, 5)
    eps, mu_inv = material_scalars(er, ur)
    plan = AssemblyPlan(field)
    e = torch.as_tensor(eps, device="cuda")
    mi = torch.as_tensor(mu_inv, device="cuda")
    E1, B1 = plan.assemble(e, mi)
    E2, B2 = plan.assemble(e, mi)
    torch.cuda.synchronize()
    assert torch.equal(torch.view_as_real(E1), torch.view_as_real(E2))
    assert torch.equal(torch.view_as_real(B1), torch.view_as_real(B2))
    # host entry point gives the same bits as the device entry point
    Eh, Bh = plan.assemble_host(eps, mu_inv)
    assert np.array_equal(Eh.view(np.float64), torch.view_as_real(E1).cpu().numpy().ravel())
    assert np.array_equal(Bh.view(np.float64), torch.view_as_real(B1).cpu().numpy().ravel())
    # page-locked outputs (the fill stores into host memory directly): same bits
    pE = torch.zeros(plan.nnz, dtype=torch.complex128, pin_memory=True)
    pB = torch.zeros(plan.nnz, dtype=torch.complex128, pin_memory=True)
    plan.assemble_host(eps, mu_inv, pE.numpy(), pB.numpy())
    assert np.array_equal(pE.numpy().view(np.float64), torch.view_as_real(E1).cpu().numpy().ravel())
    assert np.array_equal(pB.numpy().view(np.float64), torch.view_as_real(B1).cpu().numpy().ravel())


def test_empty_mesh_and_boundary_only_entities(torch_cuda):
    """A single tet: every entity has one incidence; nnz = 20*20."""
    from emerge_gb300.assembly import tet_mass_stiffness_matrices
    from emerge_gb300.mesh import Nedelec2Basis, TetMesh
    nodes = np.array([[0, 1, 0, 0], [0, 0, 1, 0], [0, 0, 0, 1]], dtype=float) * 1e-3
    m = TetMesh(nodes, np.array([[0], [1], [2], [3]]))
    field = Nedelec2Basis(m)
    er, ur = _random_materials(1, 3)
    E, B = tet_mass_stiffness_matrices(field, er, ur)
    Eo, Bo = oracle.tet_mass_stiffness_matrices(field, er, ur)
    assert E.nnz == 400
    assert rel_to_rowmax(E, Eo) <= TOL and rel_to_rowmax(B, Bo) <= TOL


def test_bad_mesh_is_rejected(torch_cuda):
    from emerge_gb300._lib import EmgError
    from emerge_gb300.assembly import AssemblyPlan
    from emerge_gb300.mesh import Nedelec2Basis, unit_cube
    m = unit_cube(2)
    field = Nedelec2Basis(m)
    field.tet_to_field = field.tet_to_field.copy()
    field.tet_to_field[3, 5] = field.n_field + 7          # out of range
    with pytest.raises(EmgError):
        AssemblyPlan(field)
    field = Nedelec2Basis(m)
    field.tet_to_field = field.tet_to_field.copy()
    field.tet_to_field[13, 2] += 1                         # mode-2 DOF no longer pairs consistently
    with pytest.raises(EmgError):
        AssemblyPlan(field)


def _random_tensors(nT, seed):
    """Full complex (3,3,nT) tensors: lossy, non-symmetric, diagonally dominant."""
    rng = np.random.default_rng(seed)
    er = (rng.uniform(-0.8, 0.8, (3, 3, nT)) + 1j * rng.uniform(-0.05, 0.05, (3, 3, nT)))
    ur = (rng.uniform(-0.3, 0.3, (3, 3, nT)) + 1j * rng.uniform(-0.02, 0.02, (3, 3, nT)))
    for k in range(3):
        er[k, k] += rng.uniform(2, 10, nT) * (1 - 1j * rng.uniform(0.001, 0.02, nT))
        ur[k, k] += rng.uniform(0.8, 3, nT)
    return er, ur


@pytest.mark.parametrize("n,kind", [(5, "full"), (7, "diagonal"), (6, "mixed")])
def test_tensor_materials_match_oracle(torch_cuda, n, kind):
    """Anisotropic er / ur (the general _matrix_builder case) through the tensor fill."""
    from emerge_gb300.assembly import tet_mass_stiffness_matrices
    from emerge_gb300.mesh import Nedelec2Basis, unit_cube
    m = unit_cube(n, jitter=0.15, seed=n)
    field = Nedelec2Basis(m)
    er, ur = _random_tensors(m.n_tets, 40 + n)
    if kind == "diagonal":           # diag(a, b, c): matinv's reciprocal branch
        er = er * np.eye(3)[:, :, None]
        ur = ur * np.eye(3)[:, :, None]
    elif kind == "mixed":            # isotropic tets next to full tensors
        iso_er, iso_ur = _random_materials(m.n_tets, n, mu_one=False)
        pick = np.arange(m.n_tets) % 3 == 0
        er[:, :, pick] = iso_er[:, :, pick]
        ur[:, :, pick] = iso_ur[:, :, pick]
    E, B = tet_mass_stiffness_matrices(field, er, ur)
    Eo, Bo = oracle.tet_mass_stiffness_matrices(field, er, ur)
    assert rel_to_rowmax(E, Eo) <= TOL
    assert rel_to_rowmax(B, Bo) <= TOL


def test_tensor_fill_of_isotropic_tensors_matches_scalar_fill(torch_cuda):
    """The tensor fill given s·I tensors agrees with the float-float scalar fill."""
    torch = torch_cuda
    from emerge_gb300.assembly import AssemblyPlan, material_scalars, matinv_tensors
    from emerge_gb300.mesh import Nedelec2Basis, unit_cube
    m = unit_cube(6, jitter=0.15, seed=3)
    field = Nedelec2Basis(m)
    er, ur = _random_materials(m.n_tets, 8, mu_one=False)
    plan = AssemblyPlan(field)
    eps, mu_inv = material_scalars(er, ur)
    E1, B1 = plan.assemble(torch.as_tensor(eps, device="cuda"), torch.as_tensor(mu_inv, device="cuda"))
    E2, B2 = plan.assemble_tensor(torch.as_tensor(er.reshape(9, -1).copy(), device="cuda"),
                                  torch.as_tensor(matinv_tensors(ur).reshape(9, -1).copy(), device="cuda"))
    Eh, Bh = plan.assemble_tensor_host(er.reshape(9, -1), matinv_tensors(ur).reshape(9, -1))
    torch.cuda.synchronize()
    ip, ix = plan.pattern_host()
    from scipy.sparse import csr_matrix
    N = plan.n_field
    mk = lambda v: csr_matrix((v, ix, ip), shape=(N, N))  # noqa: E731
    assert rel_to_rowmax(mk(E2.cpu().numpy()), mk(E1.cpu().numpy())) <= TOL
    assert rel_to_rowmax(mk(B2.cpu().numpy()), mk(B1.cpu().numpy())) <= TOL
    assert np.array_equal(Eh, E2.cpu().numpy()) and np.array_equal(Bh, B2.cpu().numpy())


def test_high_valence_edge_matches_oracle(torch_cuda):
    """An edge shared by 16 tets (beyond the float-float fill's 12) takes the FP64 fill."""
    from emerge_gb300.assembly import AssemblyPlan, tet_mass_stiffness_matrices
    from emerge_gb300.mesh import Nedelec2Basis, TetMesh
    M = 16
    ang = 2 * np.pi * np.arange(M) / M
    ring = np.stack([np.cos(ang), np.sin(ang), 0.5 + 0.1 * np.sin(3 * ang)]) * 1e-3
    nodes = np.concatenate([np.array([[0, 0], [0, 0], [0, 1e-3]]), ring], axis=1)
    tets = np.stack([np.zeros(M, int), np.ones(M, int), 2 + np.arange(M), 2 + (np.arange(M) + 1) % M])
    m = TetMesh(nodes, tets)
    field = Nedelec2Basis(m)
    er, ur = _random_materials(M, 11, mu_one=False)
    E, B = tet_mass_stiffness_matrices(field, er, ur)
    Eo, Bo = oracle.tet_mass_stiffness_matrices(field, er, ur)
    assert rel_to_rowmax(E, Eo) <= TOL
    assert rel_to_rowmax(B, Bo) <= TOL


def test_cube80_row_blocks_match_oracle(torch_cuda):
    """The assembly benchmark's own workload (80^3 Kuhn cube, 3,072,000 tets, jittered,
    random lossy eps): the float-float fill's E and B on 5000 random rows plus 2048-row
    blocks at the start, middle and end of the DOF numbering, against the oracle run on the
    tets that touch those rows.  Pattern bit-exact, values within 1e-12 of each row's
    largest entry."""
    torch = torch_cuda
    import bench
    from emerge_gb300.assembly import AssemblyPlan
    m, field, er_s = bench.make_workload(80)
    plan = AssemblyPlan(field)
    E, B = plan.assemble(torch.as_tensor(er_s, device="cuda"),
                         torch.ones(m.n_tets, dtype=torch.complex128, device="cuda"))
    p = bench.assembly_parity(field, er_s, plan, E, B)
    assert p["tets"] >= 10_000
    assert p["pattern_exact"]
    assert p["max_rel_E"] <= TOL and p["max_rel_B"] <= TOL, p


@pytest.mark.parametrize("orient", ["descending", "mixed"])
def test_edge_and_face_orientations(torch_cuda, orient):
    """Edge and face orientations other than ascending vertex ids.  ``descending``: every
    edge and face vertex list reversed, so each tet still follows one vertex order (the
    canonical-frame fill); ``mixed``: a random half of the edges reversed, so some tets
    follow no single order (the per-lane fill).  Both against the oracle, which evaluates
    the reference's element formulas with whatever orientation the mesh arrays give."""
    import types
    from emerge_gb300.assembly import tet_mass_stiffness_matrices
    from emerge_gb300.mesh import Nedelec2Basis, unit_cube
    m = unit_cube(5, jitter=0.15, seed=4)
    base = Nedelec2Basis(m)
    edges, tris = np.array(m.edges), np.array(m.tris)
    if orient == "descending":
        edges, tris = edges[::-1].copy(), tris[::-1].copy()
    else:
        flip = np.random.default_rng(2).random(edges.shape[1]) < 0.5
        edges[:, flip] = edges[::-1, flip]
    mesh = types.SimpleNamespace(nodes=m.nodes, tets=m.tets, edges=edges, tris=tris, edge_lengths=m.edge_lengths,
                                 tet_to_edge=m.tet_to_edge, tet_to_tri=m.tet_to_tri, tri_to_edge=m.tri_to_edge)
    field = types.SimpleNamespace(mesh=mesh, tet_to_field=base.tet_to_field)
    er, ur = _random_materials(m.n_tets, 8, mu_one=False)
    E, B = tet_mass_stiffness_matrices(field, er, ur)
    Eo, Bo = oracle.tet_mass_stiffness_matrices(field, er, ur)
    assert rel_to_rowmax(E, Eo) <= TOL
    assert rel_to_rowmax(B, Bo) <= TOL


def test_matinv_kernel_matches_oracle(torch_cuda):
    """emg_matinv against the oracle's matinv (fem/mth/optimized.py:440-461) on diagonal
    tensors (reciprocal diagonal), full and mixed tensors (the reference's adj * det), and
    isotropic scalars (1 / s)."""
    torch = torch_cuda
    from emerge_gb300.assembly import matinv_device
    rng = np.random.default_rng(11)
    n = 64
    s = rng.normal(size=(3, 3, n)) + 1j * rng.normal(size=(3, 3, n)) + 3 * np.eye(3)[:, :, None]
    for t in range(0, n, 4):                    # every fourth tensor diagonal
        s[:, :, t] = np.diag(np.diag(s[:, :, t]))
    s[0, 1, 1] = s[1, 0, 1] = 0                 # off-diagonal zeros in a full tensor
    got = matinv_device(torch.as_tensor(s.reshape(9, n).copy(), device="cuda")).cpu().numpy().reshape(3, 3, n)
    for t in range(n):
        ref = oracle.matinv(s[:, :, t])
        assert np.max(np.abs(got[:, :, t] - ref)) <= 1e-13 * np.max(np.abs(ref)), t
    z = rng.uniform(0.5, 3, n) * (1 - 1j * rng.uniform(0, 0.1, n))
    gz = matinv_device(torch.as_tensor(z, device="cuda")).cpu().numpy()
    assert np.max(np.abs(gz - 1 / z) / np.abs(1 / z)) <= 1e-15
