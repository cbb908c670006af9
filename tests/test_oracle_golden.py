"""The oracle against golden vectors produced by running the EMerge reference.

CPU only.  These tests pin the oracle (oracle/ned2_oracle.cpp) before it is
trusted as the checker of the CUDA path.
"""
import numpy as np
import pytest

import oracle
from _fixtures import csr_from, field_from, load, rel_to_rowmax


def test_tet_element_matrices_match_reference():
    """ned2_tet_stiff_mass (fem/mth/tet.py:854-1088), 48 tets incl. anisotropic Ms/Mm."""
    z = load("tet_elements.npz")
    for k in range(z["D"].shape[0]):
        D, F = oracle.tet_stiff_mass(z["verts"][k], z["edge_lengths"][k], z["local_edge_map"][k],
                                     z["local_tri_map"][k], z["Ms"][k], z["Mm"][k])
        for X, R in ((D, z["D"][k]), (F, z["F"][k])):
            err = np.abs(X - R).max(axis=1) / np.abs(R).max(axis=1)
            assert err.max() <= 1e-13, (k, err.max())


def test_reference_mass_matrix_is_asymmetric():
    """The reference's face-face mass block is not symmetric; the oracle keeps that."""
    z = load("tet_elements.npz")
    F = z["F"][0]
    asym = np.abs(F - F.T).max() / np.abs(F).max()
    assert asym > 1e-3
    D = z["D"][0]
    assert np.abs(D - D.T).max() / np.abs(D).max() < 1e-12


def test_tri_elements_match_reference():
    """ned2_tri_stiff_force and ned2_tri_stiff (fem/mth/tri.py:575-797)."""
    z = load("tri_elements.npz")
    for k in range(z["B_force"].shape[0]):
        B, b = oracle.tri_stiff_force(z["lcs_vertices"][k], z["gamma"][k], z["Uinc"][k], z["DPTs"])
        assert np.abs(B - z["B_force"][k]).max() <= 1e-13 * np.abs(z["B_force"][k]).max()
        assert np.abs(b - z["b_force"][k]).max() <= 1e-13 * np.abs(z["b_force"][k]).max()
        B2 = oracle.tri_stiff(z["vertices"][k], z["edge_lengths"][k], z["gamma"][k])
        assert np.abs(B2 - z["B_stiff"][k]).max() <= 1e-12 * np.abs(z["B_stiff"][k]).max()


@pytest.mark.parametrize("tag", ["a", "b"])
def test_small_assembly_matches_reference(tag):
    """tet_mass_stiffness_matrices on a jittered 2x2x2-hex box: pattern identical, values exact."""
    z = load("small_assembly.npz")
    field = field_from(z)
    E, B = oracle.tet_mass_stiffness_matrices(field, z["er_" + tag], z["ur_" + tag])
    assert rel_to_rowmax(E, csr_from(z, "E_" + tag)) <= 1e-14
    assert rel_to_rowmax(B, csr_from(z, "B_" + tag)) <= 1e-14


def test_waveguide_assembly_checksums_match_reference():
    """WR-90 guide (3264 tets): row sums and first moments of E and B from the reference."""
    z = load("waveguide.npz")
    field = field_from(z)
    nT = field.mesh.n_tets
    eye = np.repeat(np.eye(3, dtype=np.complex128)[:, :, None], nT, axis=2)
    E, B = oracle.tet_mass_stiffness_matrices(field, eye, eye)
    n = E.shape[0]
    w = (np.arange(n) + 1.0) / n
    for name, M in (("E", E), ("B", B)):
        assert M.nnz == int(z[name + "_nnz"])
        assert np.array_equal(M.indptr, z[name + "_indptr"])
        rs = np.asarray(M.sum(axis=1)).ravel()
        ref = z[name + "_rowsum"]
        scale = np.abs(M).max(axis=1).toarray().ravel()
        assert np.max(np.abs(rs - ref) / scale) <= 1e-12
        assert np.max(np.abs(M @ w - z[name + "_rowmom"]) / scale) <= 1e-12


def test_volume_rounding_matches_reference_expansion():
    """V uses the reference's expanded 24-term sum; far from the origin it differs from the
    translation-invariant value by far more than 1e-12 relative, and the oracle keeps the
    reference's rounding."""
    v = 0.9 + 0.0125 * np.array([[0, 1, 0, 0], [0, 0, 1, 0], [0, 0, 0, 1]], dtype=float)
    b, c, d, V = oracle.tet_coefficients_bcd(v)
    e = v[:, 1:] - v[:, :1]
    exact = abs(np.linalg.det(e)) / 6
    assert abs(V - exact) / exact > 1e-12      # the reference's own cancellation error
    z = load("tet_elements.npz")
    k = 3                                       # fixture tet with offset 0.9, h = 0.0125
    D, _ = oracle.tet_stiff_mass(z["verts"][k], z["edge_lengths"][k], z["local_edge_map"][k],
                                 z["local_tri_map"][k], z["Ms"][k], z["Mm"][k])
    assert np.array_equal(D, z["D"][k]) or np.abs(D - z["D"][k]).max() <= 1e-13 * np.abs(z["D"][k]).max()


def test_vectorised_matinv_matches_oracle():
    """The drop-in's per-tet matinv (host side of the tensor fill) against the oracle's."""
    from emerge_gb300.assembly import matinv_tensors
    rng = np.random.default_rng(7)
    nT = 40
    s = rng.normal(size=(3, 3, nT)) + 1j * rng.normal(size=(3, 3, nT))
    s[:, :, :10] *= np.eye(3)[:, :, None]            # the reciprocal-diagonal branch
    s[0, 2, 10] = 0.0                                   # partly zero off-diagonal: general branch
    got = matinv_tensors(s)
    for t in range(nT):
        ref = oracle.matinv(s[:, :, t])
        assert np.allclose(got[:, :, t], ref, rtol=1e-14, atol=0)


def test_mlp_oracle_gradient_by_finite_differences():
    """The MLP oracle's backward pass (the checker of the GPU training kernels) against
    central differences of its own loss, in FP64 without the bf16 roundings."""
    from oracle import mlp_oracle as mo
    rng = np.random.default_rng(0)
    in_dim, hidden, layers, out_dim, nb = 3, 16, 2, 5, 7
    K, N = mo.layer_dims(in_dim, hidden, layers, out_dim)
    npar = sum(n * k + n for k, n in zip(K, N))
    w = rng.normal(size=npar) * 0.3
    x = rng.normal(size=(nb, in_dim))
    t = rng.normal(size=(nb, out_dim))
    _, _, g = mo.forward_backward(w, x, t, in_dim, hidden, layers, out_dim, rounding=False)
    # only parameters that reach the loss (padding rows/columns carry zero gradient)
    for i in rng.choice(npar, 60, replace=False):
        e = np.zeros(npar)
        e[i] = 1e-6
        lp = mo.forward_backward(w + e, x, t, in_dim, hidden, layers, out_dim, rounding=False)[1]
        lm = mo.forward_backward(w - e, x, t, in_dim, hidden, layers, out_dim, rounding=False)[1]
        fd = (lp - lm) / 2e-6
        assert abs(fd - g[i]) <= 1e-7 + 1e-6 * abs(g[i]), (i, fd, g[i])
