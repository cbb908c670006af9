"""The patch-antenna case on a coarse grid (142,910 DOFs): lumped feed, lossy substrate,
interior PEC ground and patch, first-order absorbing air box.

The batched sweep (FP32 slab anchors + FP64 FGMRES, planar slabs along the longest
axis) is checked on the host, independently of its own residuals and S-parameter
path: SciPy forms ||K x - b|| / ||b|| with the host CSR K(k0) from the assembler
(<= 1e-9), and S11 is recomputed from x with the oracle's field interpolation along
the port's voltage line (fem/physics/edm/emfreq3d.py:752-766), |dS11| <= 1e-7.
(A SuperLU solve at this size takes about 20 minutes on the host: the 3-D air box
fills in, unlike the guides.)
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from emerge_gb300 import _build
    _build.build()
    return torch


def test_patch_sweep_solutions_and_sparameters(cuda):
    from emerge_gb300.freq import Assembler
    from emerge_gb300.geometry import patch_antenna
    from emerge_gb300.solver import FrequencySweep
    from oracle import interp_oracle
    p = patch_antenna()
    port = p.bcs[2]
    asm = Assembler()
    sw = FrequencySweep(asm, p.field, p.er, p.ur, p.bcs)
    sw.slab("axis")
    freqs = np.array([2.1e9, 2.5e9])
    r = sw.run_anchored(freqs, n_anchor=2, precision="fp32", tol=1e-11, restart=60, max_iter=600)
    assert r.residuals.max() <= 1e-10
    X = r.solutions.cpu().numpy()
    m = p.mesh
    mid, step = port.integration_line(m)
    verts = np.unique(m.tris[:, m.get_triangles(port.tags)].ravel())
    port_tets = np.flatnonzero(np.isin(m.tets, verts).any(axis=0))
    for fi, f in enumerate(freqs):
        K, b, solve_ids, pv = asm.assemble_freq_matrix(p.field, p.er, p.ur, p.bcs, f)
        x = np.zeros(K.shape[0], dtype=np.complex128)
        x[solve_ids] = X[:, fi]
        rhs = pv[1]
        res = (K @ x - rhs)[solve_ids]
        assert np.linalg.norm(res) <= 1e-9 * np.linalg.norm(rhs[solve_ids])
        Ex, Ey, Ez = interp_oracle.interpolate(mid, x, m.tets, m.tris, m.edges, m.nodes, p.field.tet_to_field,
                                               port_tets)
        V = np.sum(Ex * step[0] + Ey * step[1] + Ez * step[2])
        V0 = port.voltage
        S11 = np.sqrt((V - V0) ** 2 / (2 * port.Z0)) / np.sqrt(V0 ** 2 / (2 * port.Z0))
        assert abs(r.S[fi, 0, 0] - S11) <= 1e-7, (f, r.S[fi, 0, 0], S11)
        assert abs(S11) < 1.0
