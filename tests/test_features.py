"""Input features of the warm-start network (host code, no GPU)."""
import numpy as np


def test_feature_layout_and_fourier_count():
    """[f, sin/cos(k pi f/2) for k = 1..n_fourier, one-hot port]; default 6 harmonics,
    16 for the minimal-residual targets."""
    from emerge_gb300.mlp import N_FOURIER, features
    f = np.linspace(-1, 1, 5)
    port = np.array([0, 1, 0, 1, 1])
    for nf in (N_FOURIER, 16):
        x = features(f, port, 2, nf)
        assert x.shape == (5, 1 + 2 * nf + 2) and x.dtype == np.float32
        assert np.allclose(x[:, 0], f)
        k = 3
        assert np.allclose(x[:, 1 + 2 * (k - 1)], np.sin(k * np.pi * f / 2), atol=1e-6)
        assert np.allclose(x[:, 2 + 2 * (k - 1)], np.cos(k * np.pi * f / 2), atol=1e-6)
        assert np.array_equal(x[:, -2:], np.eye(2, dtype=np.float32)[port])
    assert features(f, port, 2).shape[1] == 1 + 2 * N_FOURIER + 2
