"""GPU solve path against the reference's SuperLU solutions and S-parameters (WR-90 guide).

Tolerances: solutions within 1e-6 relative (GMRES stops at a 1e-10 relative
residual), S-parameters within 1e-4 (linear units) of the reference.
"""
import numpy as np
import pytest

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
def waveguide(torch_cuda):
    from emerge_gb300.freq import Assembler
    z = load("waveguide.npz")
    field, bcs = waveguide_field_and_bcs(z)
    nT = field.mesh.n_tets
    eye = np.repeat(np.eye(3, dtype=np.complex128)[:, :, None], nT, axis=2)
    return z, field, bcs, eye, Assembler()


def test_gpu_solver_matches_superlu(waveguide):
    """GPUSolver through the reference SolveRoutine contract: restricted system in, solution out."""
    from emerge_gb300.solver import GPUSolver
    z, field, bcs, eye, asm = waveguide
    K, b, sid, pvs = asm.assemble_freq_matrix(field, eye, eye, bcs, float(z["freqs"][1]), cache_matrices=True)
    A = K.tocsc()[sid][:, sid]
    solver = GPUSolver(tol=1e-10)
    for pn in (1, 2):
        x_r, info = solver.solve(A, (b + pvs[pn])[sid], None, reuse_factorization=(pn == 2))
        assert info == 0
        x = np.zeros(K.shape[0], dtype=np.complex128)
        x[sid] = x_r
        ref = z[f"x1_{pn}"]
        assert np.linalg.norm(x - ref) / np.linalg.norm(ref) <= 1e-6
    assert solver.last_residual <= 1e-9


@pytest.mark.parametrize("method", ["plain", "batched"])
def test_sweep_sparams_match_reference(waveguide, method):
    from emerge_gb300.solver import FrequencySweep
    z, field, bcs, eye, asm = waveguide
    sw = FrequencySweep(asm, field, eye, eye, bcs)
    res = sw.run(z["freqs"], method=method, tol=1e-10)
    assert np.all(res.residuals <= 1e-9)
    assert np.max(np.abs(res.S - z["S"])) <= 1e-4
    # solutions against SuperLU
    X = sw.sys.scatter(res.solutions).cpu().numpy()          # (nf*np, N)
    for f in range(len(z["freqs"])):
        for p in range(2):
            ref = z[f"x{f}_{p + 1}"]
            assert np.linalg.norm(X[f * 2 + p] - ref) / np.linalg.norm(ref) <= 1e-6


def test_warm_start_sweep_agrees_and_saves_iterations(waveguide):
    """Reduced-basis warm start: same S-parameters as the plain sweep, fewer iterations."""
    from emerge_gb300.solver import FrequencySweep
    z, field, bcs, eye, asm = waveguide
    sw = FrequencySweep(asm, field, eye, eye, bcs)
    freqs = np.linspace(8.5e9, 10.5e9, 9)
    cold = sw.run(freqs, method="batched", tol=1e-10)
    warm = sw.run_warm(freqs, n_train=3, tol=1e-10)
    assert np.all(warm.residuals <= 1e-9)
    assert np.max(np.abs(warm.S - cold.S)) <= 1e-6
    assert warm.iterations.sum() < cold.iterations.sum()


def test_mlp_warm_start_gain_over_cold_start(waveguide):
    """What the trained warm-start network gains: on the frequencies it predicts (all but
    the training points) its guess leaves a several times smaller initial residual than
    the zero guess of the method without it (median ratio < 0.3; about 0.12 measured),
    and the sweep needs no more iterations there; the S-parameters agree with the cold
    sweep."""
    import torch
    from emerge_gb300.solver import FrequencySweep
    z, field, bcs, eye, asm = waveguide
    sw = FrequencySweep(asm, field, eye, eye, bcs)
    freqs = np.linspace(8.5e9, 10.5e9, 17)
    cold = sw.run_anchored(freqs, n_anchor=1, precision="fp32", tol=1e-10)
    warm = sw.run_warm(freqs, n_train=5, solver="anchored", n_anchor=1, precision="fp32", guess="mlp", tol=1e-10,
                       mlp_steps=1500)
    assert np.all(warm.residuals <= 1e-9)
    assert np.max(np.abs(warm.S - cold.S)) <= 1e-6
    assert warm.info["mlp_loss"] < 1e-2
    tr, others = warm.info["train_index"], warm.info["final_index"]
    # initial residuals of the network's guess on the predicted frequencies
    X0, _ = sw.mlp_guess(warm.solutions.reshape(sw.sys.n, len(freqs), 2)[:, tr].reshape(sw.sys.n, -1),
                         freqs[tr], freqs, steps=1500)
    k0, gam, beta = sw._coeffs(freqs)
    A = sw.sys.form(sw.E, sw.B, k0 ** 2, sw.P, gam)
    cm = torch.arange(len(freqs), dtype=torch.int32, device="cuda").repeat_interleave(2)
    b = sw._rhs(beta)
    r = sw.sys.spmv(A, X0, cm, b)
    ratio = (torch.linalg.norm(r, dim=0) / torch.linalg.norm(b, dim=0)).cpu().numpy().reshape(len(freqs), 2)
    assert np.median(ratio[others]) < 0.3
    assert warm.iterations[others].sum() <= cold.iterations[others].sum()


def test_matrix_family_product_equals_formed_matrices(waveguide):
    """A(k) X from the family (E, B, P_1, P_2) with coefficients (1, -k^2, gamma_p) equals
    the product with the formed restricted matrices (emg_rplan_form)."""
    import torch
    from emerge_gb300.solver import FrequencySweep
    z, field, bcs, eye, asm = waveguide
    sw = FrequencySweep(asm, field, eye, eye, bcs)
    freqs = np.array([8.7e9, 9.9e9, 11.3e9])
    k0, gam, beta = sw._coeffs(freqs)
    A = sw.sys.form(sw.E, sw.B, k0 ** 2, sw.P, gam)
    fam = sw.family()
    coef = np.zeros((len(freqs), fam.shape[0]), dtype=np.complex128)
    coef[:, 0], coef[:, 1], coef[:, 2:] = 1.0, -k0 ** 2, gam.T
    rng = np.random.default_rng(3)
    X = torch.as_tensor(rng.standard_normal((sw.sys.n, 3)) + 1j * rng.standard_normal((sw.sys.n, 3)), device="cuda")
    cm = torch.arange(3, dtype=torch.int32, device="cuda")
    ref = sw.sys.spmv(A, X, cm)
    got = sw.sys.spmv_family(fam, torch.as_tensor(coef, device="cuda"), X)
    assert (torch.linalg.norm(got - ref) / torch.linalg.norm(ref)).item() <= 1e-13


def test_dielectric_port_sparams_match_reference(torch_cuda):
    """A guide whose port 1 face sits in a lossy dielectric (er = 2.2 - 0.02j) and port 2 in
    air: the S-parameters carry the reference's per-triangle material weight of the mode
    integrals (fem/physics/edm/emfreq3d.py:767-778), which makes |S12 / S21| close to |er1| here.
    Sweep S against the reference's, fields against its SuperLU solutions."""
    from emerge_gb300.freq import Assembler
    from emerge_gb300.solver import FrequencySweep
    z = load("waveguide_diel.npz")
    field, bcs = waveguide_field_and_bcs(z)
    er = np.eye(3, dtype=np.complex128)[:, :, None] * z["eps"][None, None, :]
    ur = np.repeat(np.eye(3, dtype=np.complex128)[:, :, None], field.mesh.n_tets, axis=2)
    sw = FrequencySweep(Assembler(), field, er, ur, bcs)
    res = sw.run(np.array([float(z["freq"])]), method="plain", tol=1e-11)
    assert np.all(res.residuals <= 1e-10)
    X = sw.sys.scatter(res.solutions).cpu().numpy()
    for p in range(2):
        ref = z[f"x_{p + 1}"]
        assert np.linalg.norm(X[p] - ref) / np.linalg.norm(ref) <= 1e-6
    assert np.max(np.abs(res.S[0] - z["S"])) <= 1e-4
    assert abs(abs(z["S"][0, 1] / z["S"][1, 0]) - abs(2.2 - 0.02j)) < 0.05


def test_mlp_minimal_residual_targets(waveguide):
    """The network trained on the reduced system's minimal-residual coefficients (dense
    frequencies, same converged basis) leaves a smaller initial residual on the
    predicted frequencies than the zero guess (median ratio < 0.1), and the sweep needs
    fewer iterations there than from the zero guess; S-parameters agree with cold."""
    import torch
    from emerge_gb300.solver import FrequencySweep
    z, field, bcs, eye, asm = waveguide
    sw = FrequencySweep(asm, field, eye, eye, bcs)
    freqs = np.linspace(8.5e9, 10.5e9, 17)
    cold = sw.run_anchored(freqs, n_anchor=1, precision="fp32", tol=1e-10)
    warm = sw.run_warm(freqs, n_train=5, solver="anchored", n_anchor=1, precision="fp32", guess="mlp", tol=1e-10,
                       mlp_steps=1500, mlp_target="minres")
    assert np.all(warm.residuals <= 1e-9)
    assert np.max(np.abs(warm.S - cold.S)) <= 1e-6
    tr, others = warm.info["train_index"], warm.info["final_index"]
    Xs = warm.solutions.reshape(sw.sys.n, len(freqs), 2)[:, tr].reshape(sw.sys.n, -1)
    X0, loss = sw.mlp_guess(Xs, freqs[tr], freqs, steps=1500, target="minres")
    k0, gam, beta = sw._coeffs(freqs)
    A = sw.sys.form(sw.E, sw.B, k0 ** 2, sw.P, gam)
    cm = torch.arange(len(freqs), dtype=torch.int32, device="cuda").repeat_interleave(2)
    b = sw._rhs(beta)
    r = sw.sys.spmv(A, X0, cm, b)
    ratio = (torch.linalg.norm(r, dim=0) / torch.linalg.norm(b, dim=0)).cpu().numpy().reshape(len(freqs), 2)
    assert np.median(ratio[others]) < 0.1
    assert warm.iterations[others].sum() < cold.iterations[others].sum()
