"""Warm-start MLP kernels: forward and gradients against the NumPy oracle, and training."""
import numpy as np
import pytest

from oracle import mlp_oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from emerge_gb300 import _build
    _build.build()
    return torch


def test_forward_and_gradients_match_oracle(torch_cuda):
    torch = torch_cuda
    from emerge_gb300.mlp import MLP
    rng = np.random.default_rng(0)
    nin, nout, nb = 15, 20, 40
    net = MLP(nin, nout, hidden=128, layers=3, max_batch=64, seed=3)
    x = rng.uniform(-1, 1, (nb, nin)).astype(np.float32)
    t = rng.normal(0, 0.5, (nb, nout)).astype(np.float32)
    w = net.params()
    y = net.forward(torch.as_tensor(x)).cpu().numpy()
    y_ref, loss_ref, g_ref = mlp_oracle.forward_backward(w, x, t, nin, 128, 3, nout)
    assert np.linalg.norm(y - y_ref) / np.linalg.norm(y_ref) <= 2e-2
    g = net.gradients(torch.as_tensor(x), torch.as_tensor(t))
    assert abs(net.loss() - loss_ref) / loss_ref <= 2e-2
    # per-layer relative error of the gradient
    assert np.linalg.norm(g - g_ref) / np.linalg.norm(g_ref) <= 2e-2
    # the parameters did not move (lr = 0)
    assert np.array_equal(net.params(), w)


def test_training_fits_a_smooth_map(torch_cuda):
    torch = torch_cuda
    from emerge_gb300.mlp import MLP, features
    f = np.linspace(-1, 1, 32)
    x = features(np.repeat(f, 2), np.tile([0, 1], 32), 2)
    t = np.stack([np.sin(3 * np.repeat(f, 2)) + np.tile([0, 0.5], 32), np.cos(2 * np.repeat(f, 2))], axis=1)
    t = t.astype(np.float32)
    net = MLP(x.shape[1], 2, max_batch=64, seed=1)
    hist = net.fit(torch.as_tensor(x), torch.as_tensor(t), steps=1500, lr=3e-3)
    assert hist[-1] < hist[0] / 100
