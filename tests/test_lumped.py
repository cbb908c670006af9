"""LumpedPort (fem/bc.py:620-745) against the reference's own run (tests/golden/lumped.npz).

A parallel-plate line, 15 x 6 x 2 mm (1080 tets): PEC plates at z = 0 and z = 2 mm,
first-order absorbing walls at y = 0 and y = 6 mm, lumped ports (50 ohm, E along +z)
on the x = 0 and x = 15 mm faces, eps_r = 2.2 - 0.01j, 10 GHz.

CPU: the port's gamma and voltage line.  GPU: K and the port vectors (1e-12 of the
row scale), the solutions and the voltage-integral S-parameters against SuperLU's.
"""
import numpy as np
import pytest

from _fixtures import field_from, load


def _case():
    from emerge_gb300 import bc as pbc
    from emerge_gb300 import mesh as pm
    z = load("lumped.npz")
    field = field_from(z)
    L, W, H = (float(v) for v in z["dims"])
    tag_tris = {(pm.FACE_XMIN,): z["port_tris_1"], (pm.FACE_XMAX,): z["port_tris_2"],
                (pm.FACE_ZMIN, pm.FACE_ZMAX): z["pec_tris"], (pm.FACE_YMIN, pm.FACE_YMAX): z["abc_tris"]}
    field.mesh.get_triangles = lambda tags: np.asarray(tag_tris[tuple(tags)], dtype=np.int64)
    p1 = pbc.LumpedPort([pm.FACE_XMIN], 1, width=W, height=H, direction=(0, 0, 1), normal=(-1, 0, 0), Z0=50.0)
    p2 = pbc.LumpedPort([pm.FACE_XMAX], 2, width=W, height=H, direction=(0, 0, 1), normal=(1, 0, 0), Z0=50.0)
    bcs = [pbc.PEC([pm.FACE_ZMIN, pm.FACE_ZMAX]), pbc.AbsorbingBoundary([pm.FACE_YMIN, pm.FACE_YMAX]), p1, p2]
    nT = field.mesh.n_tets
    er = np.repeat(np.eye(3, dtype=np.complex128)[:, :, None], nT, axis=2) * complex(z["er"])
    ur = np.repeat(np.eye(3, dtype=np.complex128)[:, :, None], nT, axis=2)
    return z, field, bcs, er, ur


def test_port_coefficients_and_voltage_line():
    z, field, bcs, _, _ = _case()
    k0 = 2 * np.pi * float(z["freq"]) / 299792458
    for p in bcs[2:]:
        assert abs(p.get_gamma(k0) - complex(z[f"gamma_{p.port_number}"])) <= 1e-12 * abs(p.get_gamma(k0))
        mid, step = p.integration_line(field.mesh)
        assert np.allclose(mid, z[f"line_{p.port_number}_mid"], rtol=0, atol=1e-15)
        assert np.allclose(step, z[f"line_{p.port_number}_d"], rtol=0, atol=1e-15)


@pytest.fixture(scope="module")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from emerge_gb300 import _build
    _build.build()
    return torch


@pytest.mark.gpu
def test_assembled_system_matches_reference(cuda):
    from emerge_gb300.freq import Assembler
    z, field, bcs, er, ur = _case()
    K, b, solve_ids, pvecs = Assembler().assemble_freq_matrix(field, er, ur, bcs, float(z["freq"]))
    n = K.shape[0]
    scale = np.abs(K).max(axis=1).toarray().ravel()
    assert np.max(np.abs(np.asarray(K.sum(axis=1)).ravel() - z["K_rowsum"]) / scale) <= 1e-12
    assert np.max(np.abs(K @ ((np.arange(n) + 1.0) / n) - z["K_rowmom"]) / scale) <= 1e-12
    assert np.array_equal(solve_ids, z["solve_ids"])
    for pn in (1, 2):
        ref = np.zeros(n, dtype=np.complex128)
        ref[z[f"pvec_{pn}_idx"]] = z[f"pvec_{pn}_val"]
        assert np.max(np.abs(pvecs[pn] - ref)) <= 1e-12 * np.abs(ref).max()


@pytest.mark.gpu
def test_sweep_sparameters_match_reference(cuda):
    from emerge_gb300.freq import Assembler
    from emerge_gb300.solver import FrequencySweep
    z, field, bcs, er, ur = _case()
    sw = FrequencySweep(Assembler(), field, er, ur, bcs)
    r = sw.run([float(z["freq"])], method="plain", precond="slab64", tol=1e-12)
    S = r.S[0]
    assert np.max(np.abs(S - z["S"])) <= 1e-8, (S, z["S"])
    X = r.solutions.cpu().numpy()
    for j, pn in enumerate((1, 2)):
        ref = z[f"x_{pn}"][sw.solve_ids]
        assert np.linalg.norm(X[:, j] - ref) <= 1e-9 * np.linalg.norm(ref)


@pytest.mark.gpu
def test_line_weights_equal_interpolated_voltage(cuda):
    """sum w x[dofs] = sum_i dl_i . E_x(mid_i) for random solutions (the interpolation path)."""
    from emerge_gb300.field import interpolate, line_weights
    z, field, bcs, _, _ = _case()
    rng = np.random.default_rng(2)
    tets = np.arange(field.mesh.n_tets)
    for p in bcs[2:]:
        mid, step = p.integration_line(field.mesh)
        dofs, w = line_weights(field, mid, step, tetids=tets)
        dofs, w = dofs.cpu().numpy(), w.cpu().numpy()
        assert (dofs >= 0).all()
        for _ in range(3):
            x = rng.normal(size=field.n_field) + 1j * rng.normal(size=field.n_field)
            Ex, Ey, Ez = interpolate(field, x, *mid, tetids=tets)
            V = np.sum(Ex * step[0] + Ey * step[1] + Ez * step[2])
            Vw = np.sum(w * x[dofs])
            assert abs(Vw - V) <= 1e-12 * np.sum(np.abs(w * x[dofs]))


def test_port_frames_match_reference():
    """frame_from_normal against the reference's Axis.construct_cs (fem/cs.py:63-70)."""
    from emerge_gb300.bc import frame_from_normal
    z = load("frames.npz")
    for n, B in zip(z["normals"], z["bases"]):
        assert np.allclose(frame_from_normal(n)._basis, B, rtol=0, atol=1e-15), n
