"""Stratton-Chu far field: oracle against the reference's output, GPU against both.

The reference computes in complex64 (fem/physics/edm/sc.py:26-140); the oracle
in FP64 from the same FP32 inputs. Tolerance: 1e-5 of max |E_ff| (resp. |H_ff|),
about five times the reference's own complex64 rounding on this case (2e-6).
"""
import types

import numpy as np
import pytest

from _fixtures import load
from oracle import farfield_oracle as fo

TOL = 1e-5


def _case():
    z = load("farfield.npz")
    mesh = types.SimpleNamespace(n_tris=int(z["n_tris"]), tri_to_edge=z["tri_to_edge"], normals=z["normals"],
                                 areas=z["areas"], edge_centers=z["edge_centers"])
    return z, mesh


def _rel(X, R):
    return float(np.abs(X - R).max() / np.abs(R).max())


def test_oracle_matches_reference():
    z, mesh = _case()
    wns = fo.surface_weights(mesh.edge_centers.shape[1], mesh.tri_to_edge, mesh.normals, mesh.areas)
    E, H = fo.stratton_chu_ff(z["Ein"], z["Hin"], mesh.edge_centers, wns, z["theta"], z["phi"], float(z["k0"]))
    assert _rel(E, z["Eout"]) <= TOL
    assert _rel(H, z["Hout"]) <= TOL


def test_weights_match_oracle_bitwise():
    from emerge_gb300.farfield import surface_weights
    z, mesh = _case()
    a = surface_weights(mesh)
    b = fo.surface_weights(mesh.edge_centers.shape[1], mesh.tri_to_edge, mesh.normals, mesh.areas)
    assert np.array_equal(a.view(np.int32), b.view(np.int32))


@pytest.fixture(scope="module")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from emerge_gb300 import _build
    _build.build()
    return torch


@pytest.mark.gpu
def test_gpu_matches_reference_and_oracle(cuda):
    from emerge_gb300.farfield import stratton_chu
    z, mesh = _case()
    E, H = stratton_chu(z["Ein"], z["Hin"], mesh, z["theta"], z["phi"], float(z["k0"]))
    assert _rel(E, z["Eout"]) <= TOL and _rel(H, z["Hout"]) <= TOL
    wns = fo.surface_weights(mesh.edge_centers.shape[1], mesh.tri_to_edge, mesh.normals, mesh.areas)
    Eo, Ho = fo.stratton_chu_ff(z["Ein"], z["Hin"], mesh.edge_centers, wns, z["theta"], z["phi"], float(z["k0"]))
    assert _rel(E, Eo) <= TOL and _rel(H, Ho) <= TOL


@pytest.mark.gpu
def test_gpu_many_chunks_and_cutoff(cuda):
    """Several 512-source chunks, directions not a multiple of the block, sources below the cut-off."""
    from emerge_gb300.farfield import stratton_chu
    rng = np.random.default_rng(9)
    ns, nd = 2600, 1000
    tri_to_edge = rng.integers(0, ns, (3, 1500))
    normals = rng.normal(size=(3, 1500))
    normals /= np.linalg.norm(normals, axis=0)
    mesh = types.SimpleNamespace(n_tris=1500, tri_to_edge=tri_to_edge, normals=normals,
                                 areas=rng.uniform(1e-6, 4e-6, 1500), edge_centers=rng.uniform(-0.04, 0.04, (3, ns)))
    Ein = rng.normal(size=(3, ns)) + 1j * rng.normal(size=(3, ns))
    Hin = (rng.normal(size=(3, ns)) + 1j * rng.normal(size=(3, ns))) / 377
    Ein[:, :300] *= 1e-5                                   # dropped by the 1e-3 cut-off
    theta = rng.uniform(-np.pi / 2, np.pi / 2, nd)
    phi = rng.uniform(0, 2 * np.pi, nd)
    k0 = 2 * np.pi * 12e9 / 299792458
    E, H = stratton_chu(Ein, Hin, mesh, theta, phi, k0)
    wns = fo.surface_weights(ns, tri_to_edge, normals, mesh.areas)
    Eo, Ho = fo.stratton_chu_ff(Ein, Hin, mesh.edge_centers, wns, theta, phi, k0)
    assert _rel(E, Eo) <= TOL and _rel(H, Ho) <= TOL
