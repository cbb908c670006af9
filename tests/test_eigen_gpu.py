"""Cavity eigenmodes (shift-invert Arnoldi on FP32 slab factors + FP64 FGMRES)
against SciPy's ARPACK ``eigs`` on the same restricted matrices, the method of the
reference's 3-D eigenmode path (fem/physics/edm/emfreq3d.py:833-848).

Tolerance: relative eigenvalue error <= 1e-8 against ARPACK in FP64.
"""
import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from emerge_gb300 import _build
    _build.build()
    return torch


def _host(ce, vals):
    ptr, ind = ce.sys.pattern()
    n = ce.sys.n
    return sp.csc_matrix(sp.csr_matrix((vals[:, 0].cpu().numpy(), ind, ptr), shape=(n, n)))


@pytest.mark.parametrize("eps", [1.0, 12.0])
def test_cavity_modes_match_arpack(torch_cuda, eps):
    from emerge_gb300.eigen import CavityEigen, box_sigma
    from emerge_gb300.freq import Assembler
    from emerge_gb300.geometry import dielectric_cavity
    a, b, c = 14e-3, 11e-3, 9e-3
    p = dielectric_cavity(a, b, c, 2.5e-3, eps, 2e-3)
    ce = CavityEigen(Assembler(), p.field, p.er, p.ur, p.bcs)
    sigma = box_sigma((a, b, c), eps)
    res = ce.solve(6, sigma=sigma, which="LR", tol=1e-10)
    assert np.all(res.residuals <= 1e-10)
    E, B = _host(ce, ce.Er), _host(ce, ce.Br)
    ref = spla.eigs(E, k=6, M=B, sigma=sigma, which="LR", tol=1e-13)[0]
    ref = np.sort(ref.real)
    assert np.max(np.abs(res.eigenvalues.real - ref) / ref) <= 1e-8
    assert np.all(np.abs(res.eigenvalues.imag) <= 1e-8 * np.abs(res.eigenvalues.real))
    if eps == 1.0:
        # the empty box: k^2 = (m pi/a)^2 + (n pi/b)^2 + (p pi/c)^2, discretisation error only
        ana = sorted({(m * np.pi / a) ** 2 + (n * np.pi / b) ** 2 + (q * np.pi / c) ** 2
                      for m in range(4) for n in range(4) for q in range(4)
                      if (m > 0) + (n > 0) + (q > 0) >= 2})
        assert abs(res.eigenvalues.real[0] - ana[0]) / ana[0] <= 1e-2


def test_batch_of_uneven_cavities(torch_cuda):
    from emerge_gb300.eigen import eig_batch
    from emerge_gb300.geometry import dielectric_cavity
    probs = [dielectric_cavity(12e-3, 10e-3, 8e-3, 2e-3, 6.0, 2e-3),
             dielectric_cavity(16e-3, 12e-3, 9e-3, 3e-3, 20.0, 2e-3)]
    out = eig_batch(probs, nmodes=4, tol=1e-10)
    assert len(out) == 2 and out[0].info["n"] != out[1].info["n"]
    for r in out:
        assert np.all(r.residuals <= 1e-10)
        assert np.all(np.diff(r.eigenvalues.real) >= 0) and r.eigenvalues.real[0] > r.sigma
