"""tcgen05 TF32 GEMM tile (emerge_gb300/csrc/emg_tc.cu) against a PyTorch FP32 reference.

Tolerance: TF32 rounds both operands to a 10-bit mantissa, so each product carries a
relative error up to ~2^-11; with K-term sums of random-sign data the error relative to
the largest |D| stays below 5e-3 (bounded here, K <= 300).
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from emerge_gb300 import _build
    _build.build()
    return torch


@pytest.mark.parametrize("M,N,K", [(128, 64, 32), (256, 128, 96), (200, 70, 45), (300, 190, 300)])
def test_tf32_gemm_matches_fp32(torch_cuda, M, N, K):
    torch = torch_cuda
    from emerge_gb300 import _lib
    g = torch.Generator(device="cpu").manual_seed(M * 7 + N)
    A = torch.randn((M, K), generator=g).cuda()
    B = torch.randn((N, K), generator=g).cuda()
    D = torch.full((M, N), float("nan"), device="cuda")
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    _lib.call("emg_tc_gemm_tf32", M, N, K, ctypes.c_void_p(A.data_ptr()), K, ctypes.c_void_p(B.data_ptr()), K,
              ctypes.c_void_p(D.data_ptr()), N, ctypes.c_void_p(st.data_ptr()), s)
    torch.cuda.synchronize()
    assert int(st.item()) == 0
    ref = A.double() @ B.double().T
    err = ((D.double() - ref).abs().max() / ref.abs().max()).item()
    assert err < 5e-3, err
