"""2-D port modal analysis: element matrices against the reference, modes against the oracle.

Element matrices: generalized_matrix_GQ (fem/physics/edm/nedeleclegrange2.py:224-382)
run by the reference on 24 triangles (tests/golden/port_elements.npz); held to 1e-11
of each matrix's largest entry (the reference sums the 6-point rule in another order).
Modes: the WR-90 port face of the straight guide, against the same pipeline with the
oracle's element matrices and SciPy's generalized eig (the reference's LAPACK call,
fem/solver.py:316-341) to 1e-9, and against the analytic TE10 constant.
"""
import numpy as np
import pytest

from _fixtures import load
from oracle import port_oracle as po

TOL = 1e-11


def _rel(X, R):
    return float(np.abs(X - R).max() / np.abs(R).max())


def test_oracle_element_matrices_match_reference():
    z = load("port_elements.npz")
    for k in range(z["A"].shape[0]):
        A, B = po.element_matrices(z["verts"][k], z["local_edge_map"][k], z["Ms"][k], z["Mm"][k], float(z["k0"][k]))
        assert _rel(A, z["A"][k]) <= TOL, k
        assert _rel(B, z["B"][k]) <= TOL, k


def test_port_surface_dof_map():
    from emerge_gb300.geometry import straight_waveguide
    from emerge_gb300.modes import port_surface
    p = straight_waveguide(3e-3)
    port = [bc for bc in p.bcs if getattr(bc, "port_number", None) == 1][0]
    S = port_surface(p.field.mesh, p.field.mesh.get_triangles(port.tags))
    nN, nE, nT = S.node_ids.size, S.edges.shape[1], S.tris.shape[1]
    assert nN - nE + nT == 1                               # a disc: Euler characteristic 1
    assert S.n_field == 2 * nE + 2 * nT + nN + nE
    assert np.array_equal(np.sort(np.unique(S.tri_to_field)), np.arange(S.n_field))


@pytest.fixture(scope="module")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from emerge_gb300 import _build
    _build.build()
    return torch


@pytest.mark.gpu
def test_gpu_element_matrices_match_reference(cuda):
    torch = cuda
    import ctypes
    from emerge_gb300 import _lib
    z = load("port_elements.npz")
    n = z["A"].shape[0]
    xy = torch.as_tensor(np.ascontiguousarray(np.transpose(z["verts"], (1, 2, 0))), device="cuda")       # (2, 3, n)
    lem = torch.as_tensor(np.ascontiguousarray(np.transpose(z["local_edge_map"], (1, 2, 0)).astype(np.int32)),
                          device="cuda")
    Ms = torch.as_tensor(np.ascontiguousarray(z["Ms"].reshape(n, 9).T), device="cuda")
    Mm = torch.as_tensor(np.ascontiguousarray(z["Mm"].reshape(n, 9).T), device="cuda")
    vp = lambda t: ctypes.c_void_p(t.data_ptr())                                                # noqa: E731
    for k in range(n):
        A = torch.empty((1, 14, 14), dtype=torch.complex128, device="cuda")
        B = torch.empty_like(A)
        sl = lambda t: t[..., k:k + 1].contiguous()                                            # noqa: E731
        xk, lk, mk, nk = sl(xy), sl(lem), sl(Ms), sl(Mm)
        _lib.call("emg_port_element_matrices", 1, vp(xk), vp(lk), vp(mk), vp(nk), ctypes.c_double(float(z["k0"][k])),
                  0, vp(A), vp(B), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
        assert _rel(A[0].cpu().numpy(), z["A"][k]) <= TOL, k
        assert _rel(B[0].cpu().numpy(), z["B"][k]) <= TOL, k


def _oracle_modes(field, er, ur, port, pec_tags, k0, face_block):
    """The same pipeline on the host: oracle element matrices, SciPy generalized eig."""
    import scipy.linalg
    from emerge_gb300.assembly import matinv_tensors
    from emerge_gb300.modes import port_surface
    m = field.mesh
    tri_ids = np.asarray(m.get_triangles(port.tags), dtype=np.int64)
    S = port_surface(m, tri_ids)
    nodes2 = np.linalg.pinv(port.cs._basis) @ m.nodes[:, S.node_ids]
    N = S.n_field
    A = np.zeros((N, N), dtype=np.complex128)
    B = np.zeros((N, N), dtype=np.complex128)
    tet_of = m.tri_to_tet[0, tri_ids]
    for t in range(S.tris.shape[1]):
        v = np.stack([nodes2[0][S.tris[:, t]], nodes2[1][S.tris[:, t]]])
        ev = S.edges[:, S.tri_to_edge[:, t]]
        lem = np.array([[list(S.tris[:, t]).index(ev[r, e]) for e in range(3)] for r in range(2)])
        Ae, Be = po.element_matrices(v, lem, matinv_tensors(ur[:, :, tet_of[t:t + 1]])[:, :, 0],
                                     er[:, :, tet_of[t]], k0, face_block)
        f = S.tri_to_field[:, t]
        A[np.ix_(f, f)] += Ae
        B[np.ix_(f, f)] += Be
    return S, A, B


@pytest.mark.gpu
@pytest.mark.parametrize("face_block", [False, True])
def test_wr90_modes_match_oracle(cuda, face_block):
    """The reference's form gives TE10 4.9 % high (its zero face-face block); the
    integrated block gives the analytic constant."""
    from emerge_gb300.geometry import straight_waveguide
    from emerge_gb300.modes import port_modes
    import scipy.linalg
    p = straight_waveguide(3e-3)
    port = [bc for bc in p.bcs if getattr(bc, "port_number", None) == 1][0]
    pec_tags = [t for bc in p.bcs if type(bc).__name__ == "PEC" for t in bc.tags]
    k0 = 2 * np.pi * 10e9 / 299792458
    target = 0.65 * k0
    r = port_modes(p.field, p.er, p.ur, port.tags, port.cs._basis, k0, pec_tags=pec_tags, target_kz=target,
                   face_block=face_block)
    S, A, B = _oracle_modes(p.field, p.er, p.ur, port, pec_tags, k0, face_block)
    sid = r.solve_ids
    lam = scipy.linalg.eig(A[np.ix_(sid, sid)], B[np.ix_(sid, sid)], right=False)
    keep = (lam.real <= -1) & (lam.real >= -8 * target ** 2)
    beta_o = np.sqrt(-lam[keep])
    beta_o = beta_o[np.argsort(np.abs(beta_o - target))]
    assert len(r.beta) == len(beta_o) == 1
    assert np.max(np.abs(r.beta - beta_o) / np.abs(beta_o)) <= 1e-9
    te10 = np.sqrt(k0 ** 2 - (np.pi / 0.02286) ** 2)
    if face_block:
        assert abs(r.beta[0] - te10) / te10 <= 1e-5
    else:
        assert abs(r.beta[0] - 166.0238) / 166.0238 <= 1e-5


@pytest.mark.gpu
def test_port_field_interpolation_matches_reference(cuda):
    """emg_port_interp against the reference's ned2_tri_interp_full (E) and
    ned2_tri_interp_curl (the curl term of H, weighted by the diagonal of matinv(ur)) on
    random port fields of the WR-90 port face: 1e-12 of the largest value."""
    import types
    import torch
    from emerge_gb300.modes import port_field
    z = load("port_interp.npz")
    S = types.SimpleNamespace(tris=z["tris"], tri_to_field=z["tri_to_field"])
    ud = torch.as_tensor(z["diadic_diag"], device="cuda")
    E = port_field(S, z["nodes2"], z["field"], z["coords"], 0)
    H = port_field(S, z["nodes2"], z["field"], z["coords"], 1, ud, float(z["beta"]))
    assert _rel(E, z["E"]) <= 1e-12
    assert _rel(H, z["H"]) <= 1e-12


@pytest.mark.gpu
def test_modal_port_sweep_matches_rectangular_waveport(cuda):
    """ModalPort (mode solved on the port face, normalised to unit power, beta(k0) from the
    solved mode) against the analytic TE10 RectangularWaveguide on the same WR-90 mesh.
    With the integrated face block the solved TE10 constant is the analytic one, so S21
    and S11 agree to the discretisation of the mode shape."""
    from emerge_gb300.bc import ModalPort
    from emerge_gb300.freq import Assembler
    from emerge_gb300.geometry import straight_waveguide
    from emerge_gb300.solver import FrequencySweep
    p = straight_waveguide(3e-3)
    rect = [bc for bc in p.bcs if hasattr(bc, "port_number")]
    pec = [bc for bc in p.bcs if not hasattr(bc, "port_number")]
    pec_tags = [t for bc in pec for t in bc.tags]
    modal = []
    for r in rect:
        mp = ModalPort(r.tags, r.port_number, cs=r.cs)
        modes = mp.modal_analysis(p.field, p.er, p.ur, 10e9, pec_tags=pec_tags, nmodes=1, face_block=True)
        assert len(modes) == 1 and modes[0].modetype == "TE"
        te10 = np.sqrt((2 * np.pi * 10e9 / 299792458) ** 2 - (np.pi / 0.02286) ** 2)
        assert abs(modes[0].beta - te10) / te10 < 1e-4
        assert abs(abs(modes[0].power) * modes[0].norm_factor ** 2 - 1) < 1e-12
        modal.append(mp)
    freqs = np.array([9.0e9, 10.0e9, 11.0e9])
    r_rect = FrequencySweep(Assembler(), p.field, p.er, p.ur, p.bcs).run(freqs, method="plain", precond="slab64",
                                                                          tol=1e-11)
    r_modal = FrequencySweep(Assembler(), p.field, p.er, p.ur, pec + modal).run(freqs, method="plain",
                                                                                precond="slab64", tol=1e-11)
    assert np.all(r_modal.residuals <= 1e-10)
    assert np.max(np.abs(np.abs(r_modal.S) - np.abs(r_rect.S))) <= 2e-3
    assert np.all(np.abs(np.abs(r_modal.S[:, 1, 0]) - 1) <= 5e-3)
