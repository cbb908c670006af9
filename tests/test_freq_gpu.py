"""GPU frequency-matrix assembly (K, port vectors, solve_ids) against the reference run.

The waveguide fixture holds the reference's K row sums / first moments at 9 and
10 GHz, its waveport forcing vectors and solve_ids (fem/physics/edm/assembler.py:312-388).
"""
import numpy as np
import pytest

import oracle
from _fixtures import load, waveguide_field_and_bcs

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


def test_waveguide_frequency_matrices_match_reference(torch_cuda):
    from emerge_gb300.freq import Assembler
    z = load("waveguide.npz")
    field, bcs = waveguide_field_and_bcs(z)
    nT = field.mesh.n_tets
    eye = np.repeat(np.eye(3, dtype=np.complex128)[:, :, None], nT, axis=2)
    asm = Assembler()
    for fi, f in enumerate(z["freqs"]):
        K, b, solve_ids, pvs = asm.assemble_freq_matrix(field, eye, eye, bcs, float(f), cache_matrices=True)
        n = K.shape[0]
        w = (np.arange(n) + 1.0) / n
        scale = np.abs(K).max(axis=1).toarray().ravel()
        scale[scale == 0] = 1.0
        assert np.max(np.abs(np.asarray(K.sum(axis=1)).ravel() - z[f"K{fi}_rowsum"]) / scale) <= TOL
        assert np.max(np.abs(K @ w - z[f"K{fi}_rowmom"]) / scale) <= TOL
        assert np.array_equal(solve_ids, z["solve_ids"])
        assert not np.any(b)
        for pn in (1, 2):
            ref = np.zeros(n, dtype=np.complex128)
            ref[z[f"pvec{fi}_{pn}_idx"]] = z[f"pvec{fi}_{pn}_val"]
            assert np.max(np.abs(pvs[pn] - ref)) <= TOL * np.max(np.abs(ref))


def test_abc_blocks_match_oracle(torch_cuda):
    """emg_tri_robin_abc against the oracle's ned2_tri_stiff on the reference fixture triangles."""
    torch = torch_cuda
    import ctypes
    from emerge_gb300 import _lib
    t = load("tri_elements.npz")
    V = t["vertices"]                       # (n, 3, 3): coordinate rows, vertex columns
    n = V.shape[0]
    xyz = torch.as_tensor(np.ascontiguousarray(np.transpose(V, (1, 2, 0))), device="cuda")
    el = torch.as_tensor(np.ascontiguousarray(t["edge_lengths"].T), device="cuda")
    g = complex(t["gamma"][0])
    out = torch.empty(n * 64, dtype=torch.complex128, device="cuda")
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    _lib.call("emg_tri_robin_abc", n, ctypes.c_void_p(xyz.data_ptr()), ctypes.c_void_p(el.data_ptr()),
              ctypes.c_double(g.real), ctypes.c_double(g.imag), ctypes.c_void_p(out.data_ptr()), st)
    got = out.cpu().numpy().reshape(n, 8, 8)
    for k in range(n):
        ref = oracle.tri_stiff(V[k], t["edge_lengths"][k], g)
        assert np.abs(got[k] - ref).max() <= 1e-12 * np.abs(ref).max()


def test_waveport_blocks_match_reference(torch_cuda):
    """emg_tri_robin_force against the reference's ned2_tri_stiff_force fixture (per triangle)."""
    torch = torch_cuda
    import ctypes
    from emerge_gb300 import _lib
    t = load("tri_elements.npz")
    LV = t["lcs_vertices"]                  # (n, 3, 3)
    n = LV.shape[0]
    D = t["DPTs"]
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for k in range(n):
        lcs = torch.as_tensor(np.ascontiguousarray(LV[k][:2][:, :, None]), device="cuda")           # (2, 3, 1)
        U = torch.as_tensor(np.ascontiguousarray(t["Uinc"][k][:, :, None]), device="cuda")          # (3, 6, 1)
        Dd = torch.as_tensor(np.ascontiguousarray(D), device="cuda")
        Bo = torch.empty(64, dtype=torch.complex128, device="cuda")
        bo = torch.empty(8, dtype=torch.complex128, device="cuda")
        g = complex(t["gamma"][k])
        _lib.call("emg_tri_robin_force", 1, ctypes.c_void_p(lcs.data_ptr()), ctypes.c_void_p(U.data_ptr()),
                  ctypes.c_void_p(Dd.data_ptr()), D.shape[1], ctypes.c_double(g.real), ctypes.c_double(g.imag),
                  ctypes.c_void_p(Bo.data_ptr()), ctypes.c_void_p(bo.data_ptr()), st)
        B = Bo.cpu().numpy().reshape(8, 8)
        b = bo.cpu().numpy()
        assert np.abs(B - t["B_force"][k]).max() <= 1e-12 * np.abs(t["B_force"][k]).max()
        assert np.abs(b - t["b_force"][k]).max() <= 1e-12 * np.abs(t["b_force"][k]).max()


def test_absorbing_boundary_matrix_matches_reference(torch_cuda):
    """WR-90 guide with an AbsorbingBoundary on the far end (ned2_tri_stiff path)."""
    from emerge_gb300 import bc as pbc
    from emerge_gb300 import mesh as pm
    from emerge_gb300.freq import Assembler
    from _fixtures import field_from
    z = load("waveguide_abc.npz")
    field = field_from(z)
    a, b, L = (float(v) for v in z["dims"])
    tag_tris = {(pm.FACE_YMIN,): z["port_tris_1"], (pm.FACE_YMAX,): z["abc_tris"],
                (pm.FACE_XMIN, pm.FACE_XMAX, pm.FACE_ZMIN, pm.FACE_ZMAX): z["pec_tris"]}
    field.mesh.get_triangles = lambda tags: np.asarray(tag_tris[tuple(tags)], dtype=np.int64)
    p1 = pbc.RectangularWaveguide([pm.FACE_YMIN], 1, pbc.CoordinateSystem([1.0, 0, 0], [0, 0, 1.0], [0, -1.0, 0],
                                                                        [a / 2, 0.0, b / 2]), (a, b))
    bcs = [pbc.PEC([pm.FACE_XMIN, pm.FACE_XMAX, pm.FACE_ZMIN, pm.FACE_ZMAX]), p1,
           pbc.AbsorbingBoundary([pm.FACE_YMAX])]
    nT = field.mesh.n_tets
    eye = np.repeat(np.eye(3, dtype=np.complex128)[:, :, None], nT, axis=2)
    K, b, solve_ids, pvs = Assembler().assemble_freq_matrix(field, eye, eye, bcs, float(z["freq"]))
    n = K.shape[0]
    scale = np.abs(K).max(axis=1).toarray().ravel()
    scale[scale == 0] = 1.0
    assert np.max(np.abs(np.asarray(K.sum(axis=1)).ravel() - z["K_rowsum"]) / scale) <= TOL
    assert np.max(np.abs(K @ ((np.arange(n) + 1.0) / n) - z["K_rowmom"]) / scale) <= TOL
    assert np.array_equal(solve_ids, z["solve_ids"])
    ref = np.zeros(n, dtype=np.complex128)
    ref[z["pvec_1_idx"]] = z["pvec_1_val"]
    assert np.max(np.abs(pvs[1] - ref)) <= TOL * np.max(np.abs(ref))


def test_waveguide_k_entries_match_reference(torch_cuda):
    """K(k0) at 10 GHz entry by entry against the reference's own K on the rows of the
    port faces (where the Robin blocks land) and 1500 random rows.  The reference's
    ``E - B*k0**2`` drops exact zeros (scipy binop), so every reference entry must be
    found in our pattern within 1e-12 of its row's largest entry, and every entry of ours
    outside the reference pattern must be exactly zero."""
    from emerge_gb300.freq import Assembler
    z = load("waveguide.npz")
    k = load("waveguide_k.npz")
    field, bcs = waveguide_field_and_bcs(z)
    nT = field.mesh.n_tets
    eye = np.repeat(np.eye(3, dtype=np.complex128)[:, :, None], nT, axis=2)
    K, _, _, _ = Assembler().assemble_freq_matrix(field, eye, eye, bcs, float(k["freq"]))
    K = K.tocsr()
    rows, ip, ix, dv = k["rows"], k["indptr"], k["indices"], k["data"]
    assert len(rows) > 2000 and len(np.intersect1d(rows, k["port_rows"])) == len(k["port_rows"])
    worst = 0.0
    for r_i, r in enumerate(rows):
        ref_c, ref_v = ix[ip[r_i]:ip[r_i + 1]], dv[ip[r_i]:ip[r_i + 1]]
        our_c = K.indices[K.indptr[r]:K.indptr[r + 1]]
        our_v = K.data[K.indptr[r]:K.indptr[r + 1]]
        pos = np.searchsorted(our_c, ref_c)
        assert np.all(pos < len(our_c)) and np.array_equal(our_c[pos], ref_c), f"row {r}: pattern"
        scale = max(np.abs(ref_v).max(), 1e-300)
        worst = max(worst, float(np.abs(our_v[pos] - ref_v).max() / scale))
        extra = np.ones(len(our_c), dtype=bool)
        extra[pos] = False
        assert not np.any(our_v[extra]), f"row {r}: nonzero entry outside the reference pattern"
    assert worst <= TOL, worst
