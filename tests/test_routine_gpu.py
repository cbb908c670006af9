"""The solve-routine and eigensolver drop-ins (fem/solver.py:117-131, 361-505).

``GPUSweepRoutine`` is driven exactly as ``Electrodynamics3D.frequency_domain`` drives
``physics.solveroutine`` (fem/physics/edm/emfreq3d.py:686-697): one ``solve(K, b +
port_vector, solve_ids, reuse)`` per (frequency, port), ports in boundary-condition
order, ``reuse`` False on the first port of each frequency.  Solutions within 1e-6 of
the reference's SuperLU fields.  ``GPUEigSolver`` against SciPy's dense generalized eig
with the reference's mode filter (the LAPACK slot) and against the dense eigenvalue
nearest the shift (the ARPACK slot) on the WR-90 port problem.
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


def _replay(routine, asm, field, eye, bcs, freqs, ports):
    out = {}
    for fi, f in enumerate(freqs):
        K, b, sid, pvs = asm.assemble_freq_matrix(field, eye, eye, bcs, float(f), cache_matrices=True)
        reuse = False
        for bc in ports:
            out[(fi, bc.port_number)] = routine.solve(K, b + pvs[bc.port_number], sid, reuse=reuse)
            reuse = True
    return out, K, b, sid, pvs


@pytest.mark.parametrize("method", ["warm", "anchored"])
def test_sweep_routine_replays_reference_call_sequence(torch_cuda, method):
    from emerge_gb300.freq import Assembler
    from emerge_gb300.routine import GPUSweepRoutine
    z = load("waveguide.npz")
    field, bcs = waveguide_field_and_bcs(z)
    nT = field.mesh.n_tets
    eye = np.repeat(np.eye(3, dtype=np.complex128)[:, :, None], nT, axis=2)
    freqs = z["freqs"]
    ports = [bc for bc in bcs if hasattr(bc, "port_number")]
    kw = {"n_train": 2} if method == "warm" else {}
    routine = GPUSweepRoutine(field=field, er=eye, ur=eye, bcs=bcs, frequencies=freqs, method=method, **kw)
    out, K, b, sid, pvs = _replay(routine, Assembler(), field, eye, bcs, freqs, ports)
    for (fi, pn), x in out.items():
        ref = z[f"x{fi}_{pn}"]
        assert np.linalg.norm(x - ref) / np.linalg.norm(ref) <= 1e-6, (fi, pn)
        assert not np.any(x[np.setdiff1d(np.arange(len(x)), sid)])
    assert routine.stats["served"] == 4 and routine.stats["solved_alone"] == 0
    assert routine.stats["max_check_residual"] <= 1e-8
    # a call that is not a column of the sweep (a changed matrix) is solved on its own
    x = routine.solve(K * 1.001, b + pvs[1], sid, reuse=False)
    r = (K * 1.001 @ x)[sid] - (b + pvs[1])[sid]
    assert np.linalg.norm(r) / np.linalg.norm((b + pvs[1])[sid]) <= 1e-8
    assert routine.stats["solved_alone"] == 1


def _port_problem(k0):
    from emerge_gb300.geometry import straight_waveguide
    from emerge_gb300.modes import port_problem
    p = straight_waveguide(3e-3)
    port = [bc for bc in p.bcs if getattr(bc, "port_number", None) == 1][0]
    pec_tags = [t for bc in p.bcs if type(bc).__name__ == "PEC" for t in bc.tags]
    return port_problem(p.field, p.er, p.ur, port.tags, port.cs._basis, k0, pec_tags=pec_tags)


def test_eig_solver_direct_slot_matches_lapack_filter(torch_cuda):
    """The LAPACK slot: every generalized eigenpair, filtered and ordered as
    filter_real_modes (fem/solver.py:34-68) with er_max = ur_max = 2."""
    import scipy.linalg
    import scipy.sparse as sp
    from emerge_gb300.routine import GPUEigSolver
    k0 = 2 * np.pi * 10e9 / 299792458
    pp = _port_problem(k0)
    A, B = pp.A.cpu().numpy(), pp.B.cpu().numpy()
    t = pp.target_kz
    lam_g, vec_g = GPUEigSolver(iterative=False).eig(sp.csr_matrix(A), sp.csr_matrix(B), 6, t, "LM")
    lam = scipy.linalg.eig(A, B, right=False)
    keep = (lam.real <= -1) & (lam.real >= -(t ** 2) * 8)
    lam = lam[keep]
    lam = lam[np.argsort(np.abs(np.sqrt(-lam) - t))]
    assert len(lam_g) == len(lam) >= 1
    assert np.max(np.abs(lam_g - lam) / np.abs(lam)) <= 1e-9
    for i in range(len(lam_g)):                       # each returned vector is an eigenvector
        v = vec_g[:, i]
        assert np.linalg.norm(A @ v - lam_g[i] * (B @ v)) <= 1e-8 * np.linalg.norm(A @ v)


def test_eig_solver_iterative_slot_nearest_eigenvalue(torch_cuda):
    """The ARPACK slot: the eigenvalue nearest sigma = -target_k0^2, against the dense
    generalized eigenvalues of the same pencil (TE10; the next nearest ones are the
    pencil's degenerate zero eigenvalues).  SciPy's ARPACK shift-invert is not the check
    here: on this pencil it returns complex values that are not eigenvalues of it."""
    import scipy.linalg
    import scipy.sparse as sp
    from emerge_gb300.routine import GPUEigSolver
    k0 = 2 * np.pi * 10e9 / 299792458
    pp = _port_problem(k0)
    Ad, Bd = pp.A.cpu().numpy(), pp.B.cpu().numpy()
    A, B = sp.csr_matrix(Ad), sp.csr_matrix(Bd)
    t = pp.target_kz
    lam_g, vec_g = GPUEigSolver(iterative=True).eig(A, B, 1, t, "LM")
    lam = scipy.linalg.eig(Ad, Bd, right=False)
    lam = lam[np.isfinite(lam)]
    near = lam[np.argmin(np.abs(lam + t * t))]
    assert len(lam_g) == 1 and lam_g[0] < -1
    assert abs(lam_g[0] - near.real) / abs(near.real) <= 1e-8
    v = vec_g[:, 0]
    assert np.linalg.norm(A @ v - lam_g[0] * (B @ v)) <= 1e-8 * np.linalg.norm(A @ v)
