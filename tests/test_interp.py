"""Field interpolation (ned2_tet_interp, fem/mth/tet.py:372-497): the oracle against the
reference's own values (tests/golden/interp.npz: the WR-90 guide's 10 GHz SuperLU
field at the port-1 quadrature points and at random interior points), and the GPU
kernel against the same values.  Tolerance: 1e-12 relative to the largest |E|."""
import numpy as np
import pytest

from _fixtures import field_from, load


def _mesh(z):
    i8 = lambda k: np.asarray(z[k], dtype=np.int64)  # noqa: E731
    return i8("tets"), i8("tris"), i8("edges"), np.asarray(z["nodes"]), i8("tet_to_field")


@pytest.mark.parametrize("kind", ["port", "inner"])
def test_oracle_matches_reference_interpolation(kind):
    from oracle.interp_oracle import interpolate
    z, g = load("waveguide.npz"), load("interp.npz")
    tets, tris, edges, nodes, t2f = _mesh(z)
    tetids = g["port_tets"] if kind == "port" else np.arange(tets.shape[1])
    E = np.stack(interpolate(g[f"{kind}_points"], z["x1_1"], tets, tris, edges, nodes, t2f, tetids))
    R = g[f"{kind}_E"]
    assert np.abs(E - R).max() <= 1e-12 * np.abs(R).max()


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["port", "inner"])
def test_gpu_interpolation_matches_reference(kind):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from emerge_gb300 import _build
    from emerge_gb300.field import interpolate
    _build.build()
    z, g = load("waveguide.npz"), load("interp.npz")
    field = field_from(z)
    field.mesh.tris = np.asarray(z["tris"], dtype=np.int64)
    tetids = g["port_tets"] if kind == "port" else None
    P = g[f"{kind}_points"]
    E = np.stack(interpolate(field, z["x1_1"], P[0], P[1], P[2], tetids=tetids))
    R = g[f"{kind}_E"]
    assert np.abs(E - R).max() <= 1e-12 * np.abs(R).max()
    # a point outside every searched tet gives zero
    far = interpolate(field, z["x1_1"], [1.0], [1.0], [1.0], tetids=tetids)
    assert all(abs(c[0]) == 0 for c in far)
