"""Slab (block-tridiagonal) factorization against SciPy's SuperLU, the reference's
default direct solver (fem/solver.py:248-275), on the WR-90 guide fixture.

Tolerances: FP64 factor solves within 1e-9 relative of SuperLU; FGMRES with FP32
factors converges to a 1e-10 FP64 residual and then matches SuperLU within 1e-7.
"""
import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from _fixtures import load, waveguide_field_and_bcs

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from emerge_gb300 import _build
    _build.build()
    return torch


@pytest.fixture(scope="module")
def system(torch_cuda):
    """Restricted K(f) at the fixture's two frequencies, on the device and on the host."""
    torch = torch_cuda
    from emerge_gb300.freq import Assembler
    from emerge_gb300.solver import RestrictedSystem, SlabFactor
    z = load("waveguide.npz")
    field, bcs = waveguide_field_and_bcs(z)
    nT = field.mesh.n_tets
    eye = np.repeat(np.eye(3, dtype=np.complex128)[:, :, None], nT, axis=2)
    asm = Assembler()
    Ks, rhs = [], []
    for fi in range(2):
        K, b, sid, pvs = asm.assemble_freq_matrix(field, eye, eye, bcs, float(z["freqs"][fi]), cache_matrices=True)
        Kr = sp.csr_matrix(K.tocsc()[sid][:, sid])
        Kr.sort_indices()
        Ks.append(Kr)
        rhs.append(np.stack([(b + pvs[p])[sid] for p in (1, 2)], axis=1))
    K0 = Ks[0]
    n = K0.shape[0]
    dev = torch.device("cuda")
    sysr = RestrictedSystem(torch.as_tensor(K0.indptr.astype(np.int64), device=dev),
                            torch.as_tensor(K0.indices.astype(np.int32), device=dev), K0.nnz, np.arange(n))
    vals = torch.stack([torch.as_tensor(K.data, device=dev) for K in Ks], dim=1).contiguous()   # (nnz, 2)
    slab = SlabFactor(sysr)
    return torch, sysr, slab, Ks, rhs, vals


def test_slabs_are_block_tridiagonal(system):
    torch, sysr, slab, Ks, rhs, vals = system
    off, perm = slab.levels()
    info = slab.info()
    n = Ks[0].shape[0]
    assert off[0] == 0 and off[-1] == n and np.all(np.diff(off) > 0)
    assert np.array_equal(np.sort(perm), np.arange(n))
    lev = np.empty(n, dtype=np.int64)
    lev[perm] = np.repeat(np.arange(len(off) - 1), np.diff(off))
    coo = Ks[0].tocoo()
    assert np.max(np.abs(lev[coo.row] - lev[coo.col])) <= 1
    assert info["slabs"] == len(off) - 1
    assert info["max_width"] == np.max(np.diff(off))


def test_fp64_slab_solve_matches_superlu(system):
    torch, sysr, slab, Ks, rhs, vals = system
    slab.factor(vals, [0, 1], "fp64")
    assert slab.info()["factors"] == 2
    assert slab.info()["perturbed_pivots"] == 0
    # columns: (f0, port1), (f0, port2), (f1, port1), (f1, port2)
    B = np.concatenate(rhs, axis=1)
    X = slab.apply(torch.as_tensor(B, device="cuda"), [0, 0, 1, 1]).cpu().numpy()
    for c in range(4):
        ref = spla.spsolve(Ks[c // 2].tocsc(), B[:, c])
        assert np.linalg.norm(X[:, c] - ref) / np.linalg.norm(ref) <= 1e-9


def test_fp32_factors_with_fgmres_reach_fp64_accuracy(system):
    torch, sysr, slab, Ks, rhs, vals = system
    slab.factor(vals, [0, 1], "fp32")
    B = np.concatenate(rhs, axis=1)
    Bt = torch.as_tensor(B, device="cuda")
    # the FP32 factor alone is a preconditioner, not a solve
    X32 = slab.apply(Bt, [0, 0, 1, 1]).cpu().numpy()
    ref = [spla.spsolve(Ks[c // 2].tocsc(), B[:, c]) for c in range(4)]
    e32 = max(np.linalg.norm(X32[:, c] - ref[c]) / np.linalg.norm(ref[c]) for c in range(4))
    assert 1e-8 < e32 < 0.5
    # FGMRES in FP64 around it; column 3 uses the other frequency's factor
    cmat = torch.tensor([0, 0, 1, 1], dtype=torch.int32, device="cuda")
    x, its, res = slab.gmres(vals, Bt, cmat, [0, 0, 1, 0], tol=1e-10, restart=40, max_iter=400)
    assert np.all(res <= 1e-10)
    assert np.all(its <= 60)
    x = x.cpu().numpy()
    for c in range(4):
        assert np.linalg.norm(x[:, c] - ref[c]) / np.linalg.norm(ref[c]) <= 1e-7


def test_gpusolver_slab_matches_reference(torch_cuda):
    from emerge_gb300.freq import Assembler
    from emerge_gb300.solver import GPUSolver
    z = load("waveguide.npz")
    field, bcs = waveguide_field_and_bcs(z)
    nT = field.mesh.n_tets
    eye = np.repeat(np.eye(3, dtype=np.complex128)[:, :, None], nT, axis=2)
    K, b, sid, pvs = Assembler().assemble_freq_matrix(field, eye, eye, bcs, float(z["freqs"][1]), cache_matrices=True)
    A = K.tocsc()[sid][:, sid]
    solver = GPUSolver(tol=1e-12, method="slab")
    for pn in (1, 2):
        x_r, info = solver.solve(A, (b + pvs[pn])[sid], None, reuse_factorization=(pn == 2))
        assert info == 0
        x = np.zeros(K.shape[0], dtype=np.complex128)
        x[sid] = x_r
        ref = z[f"x1_{pn}"]
        assert np.linalg.norm(x - ref) / np.linalg.norm(ref) <= 1e-9
    assert solver.last_iterations <= 3


def test_anchored_sweep_matches_reference_sparams(torch_cuda):
    from emerge_gb300.freq import Assembler
    from emerge_gb300.solver import FrequencySweep
    z = load("waveguide.npz")
    field, bcs = waveguide_field_and_bcs(z)
    nT = field.mesh.n_tets
    eye = np.repeat(np.eye(3, dtype=np.complex128)[:, :, None], nT, axis=2)
    sw = FrequencySweep(Assembler(), field, eye, eye, bcs)
    freqs = z["freqs"]
    res = sw.run_anchored(freqs, n_anchor=1, precision="fp32", tol=1e-10)
    assert np.all(res.residuals <= 1e-9)
    assert np.max(np.abs(res.S - z["S"])) <= 1e-4
    plain = sw.run(freqs, method="plain", precond="slab64", tol=1e-10)
    assert np.all(plain.residuals <= 1e-9)
    assert np.max(np.abs(plain.S - z["S"])) <= 1e-4
    assert np.max(np.abs(res.S - plain.S)) <= 1e-7


def test_wide_column_groups_use_tiled_product(system):
    """Groups of >= 48 columns take the 64 x 64 tiled product; same result as narrow groups."""
    torch, sysr, slab, Ks, rhs, vals = system
    slab.factor(vals, [0, 1], "fp64")
    rng = np.random.default_rng(5)
    n = Ks[0].shape[0]
    B = rng.standard_normal((n, 70)) + 1j * rng.standard_normal((n, 70))
    Bt = torch.as_tensor(B, device="cuda")
    wide = slab.apply(Bt, [0] * 60 + [1] * 10).cpu().numpy()
    narrow = np.concatenate([slab.apply(Bt[:, c0:c0 + 10], [0] * 10 if c0 < 60 else [1] * 10).cpu().numpy()
                             for c0 in range(0, 70, 10)], axis=1)
    assert np.max(np.abs(wide - narrow)) <= 1e-9 * np.max(np.abs(narrow))
    for c in (0, 59, 65):
        ref = spla.spsolve(Ks[0 if c < 60 else 1].tocsc(), B[:, c])
        assert np.linalg.norm(wide[:, c] - ref) / np.linalg.norm(ref) <= 1e-9


def test_mixed_precision_refinement_reaches_fp64_accuracy(system):
    """FP64 iterative refinement around FGMRES on complex FP32 vectors (FP32 factors,
    FP32 copy of A): FP64 residual 1e-10 and SuperLU's solution within 1e-7."""
    torch, sysr, slab, Ks, rhs, vals = system
    slab.factor(vals, [0, 1], "fp32")
    B = np.concatenate(rhs, axis=1)
    Bt = torch.as_tensor(B, device="cuda")
    cmat = torch.tensor([0, 0, 1, 1], dtype=torch.int32, device="cuda")
    x, its, res, steps = slab.gmres_mixed(vals, Bt, cmat, [0, 0, 1, 0], tol=1e-10, restart=40, max_iter=400)
    assert np.all(res <= 1e-10)
    assert 2 <= steps <= 6
    x = x.cpu().numpy()
    for c in range(4):
        ref = spla.spsolve(Ks[c // 2].tocsc(), B[:, c])
        assert np.linalg.norm(x[:, c] - ref) / np.linalg.norm(ref) <= 1e-7


def test_tensor_core_slab_products(system):
    """Wide-group products of an FP32-factor solve on the tcgen05 tensor cores (TF32):
    within TF32 rounding of the CUDA-core result, and FGMRES still reaches 1e-10."""
    torch, sysr, slab, Ks, rhs, vals = system
    slab.factor(vals, [0, 1], "fp32")
    rng = np.random.default_rng(11)
    n = Ks[0].shape[0]
    B = rng.standard_normal((n, 70)) + 1j * rng.standard_normal((n, 70))
    Bt = torch.as_tensor(B, device="cuda")
    cf = [0] * 60 + [1] * 10
    slab.set_tensor_cores(False)
    ref = slab.apply(Bt, cf).cpu().numpy()
    slab.set_tensor_cores(True)
    try:
        got = slab.apply(Bt, cf).cpu().numpy()
        err = np.linalg.norm(got - ref, axis=0) / np.linalg.norm(ref, axis=0)
        assert np.max(err) < 3e-2 and np.median(err) < 1e-2
        cmat = torch.zeros(60, dtype=torch.int32, device="cuda")
        x, its, res = slab.gmres(vals, Bt[:, :60].contiguous(), cmat, [0] * 60, tol=1e-10, restart=40, max_iter=400)
        assert np.all(res <= 1e-10)
    finally:
        slab.set_tensor_cores(False)


def test_autotune_picks_a_layout_and_solves_stay_exact(system):
    torch, sysr, slab, Ks, rhs, vals = system
    slab.factor(vals, [0, 1], "fp64")
    cf = [0] * 24 + [1] * 8
    out = slab.autotune(32, cf, repeats=1, candidates=[(8, 1), (8, 4), (1 << 30, 8)])
    assert set(out["choice"]) == {"wide", "max_splits"} and len(out["times_ms"]) == 3
    B = np.concatenate(rhs, axis=1)
    X = slab.apply(torch.as_tensor(B, device="cuda"), [0, 0, 1, 1]).cpu().numpy()
    for c in range(4):
        ref = spla.spsolve(Ks[c // 2].tocsc(), B[:, c])
        assert np.linalg.norm(X[:, c] - ref) / np.linalg.norm(ref) <= 1e-9
    slab.set_wide_group(8)
    slab.set_max_splits(8)


def test_tensor_core_factor_update_matches_cuda_core_fp32(system):
    """The split-TF32 tcgen05 rank-64 update gives FP32-equivalent factors: the
    preconditioned solve is as close to SuperLU as with the CUDA-core FP32 update, and
    FGMRES needs no more iterations."""
    torch, sysr, slab, Ks, rhs, vals = system
    assert slab.info()["max_width"] > 128          # several tile steps per slab
    B = np.concatenate(rhs, axis=1)
    Bt = torch.as_tensor(B, device="cuda")
    ref = [spla.spsolve(Ks[c // 2].tocsc(), B[:, c]) for c in range(4)]
    cmat = torch.tensor([0, 0, 1, 1], dtype=torch.int32, device="cuda")
    out = {}
    for on in (False, True):
        slab.set_factor_tensor_cores(on)
        slab.factor(vals, [0, 1], "fp32")
        X = slab.apply(Bt, [0, 0, 1, 1]).cpu().numpy()
        err = max(np.linalg.norm(X[:, c] - ref[c]) / np.linalg.norm(ref[c]) for c in range(4))
        x, its, res = slab.gmres(vals, Bt, cmat, [0, 0, 1, 0], tol=1e-10, restart=40, max_iter=400)
        assert np.all(res <= 1e-10)
        out[on] = (X, err, its)
    slab.set_factor_tensor_cores(True)
    X0, e0, it0 = out[False]
    X1, e1, it1 = out[True]
    assert e1 <= 3 * e0 + 1e-12
    assert np.max(np.abs(X1 - X0)) <= 10 * e0 * np.max(np.abs(X0))
    assert np.all(np.asarray(it1) <= np.asarray(it0) + 1)


def test_narrow_tiled_product_matches_row_product_fp32(system):
    """Groups of 8-16 columns take the 128 x 16 tiled product (split over K); on FP32
    factors it agrees with the warp-per-row product to FP32 rounding."""
    torch, sysr, slab, Ks, rhs, vals = system
    slab.factor(vals, [0, 1], "fp32")
    rng = np.random.default_rng(7)
    n = Ks[0].shape[0]
    B = rng.standard_normal((n, 24)) + 1j * rng.standard_normal((n, 24))
    Bt = torch.as_tensor(B, device="cuda")
    cfac = [0] * 12 + [1] * 12
    tiled = slab.apply(Bt, cfac).cpu().numpy()
    slab.set_wide_group(1 << 30)
    try:
        rows = slab.apply(Bt, cfac).cpu().numpy()
    finally:
        slab.set_wide_group(8)
    assert np.max(np.abs(tiled - rows)) <= 1e-3 * np.max(np.abs(rows))
