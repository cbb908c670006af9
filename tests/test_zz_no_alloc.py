"""emg_csr_pattern_noalloc: the CSR pattern for callers that cannot allocate.

Some host applications cannot call cudaMalloc (their device memory belongs to
another allocator, or cudaMalloc's implicit synchronisation is not allowed in
their loop).  emg_csr_pattern_noalloc builds the assembly pattern with its
scratch in a fixed array inside the library.  This test calls it through the C
ABI twice in a row, on two different meshes, and checks both results against
the plan-based entry point (emg_plan_create + emg_plan_pattern), which must
agree exactly (the pattern is integer data).  The file is named so that pytest
collects it last.
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


def _noalloc_pattern(torch, field):
    from emerge_gb300 import _lib
    nT = field.mesh.n_tets
    N = field.n_field
    t2f = torch.as_tensor(np.ascontiguousarray(field.tet_to_field, dtype=np.int32), device="cuda")
    indptr = torch.full((N + 1,), -1, dtype=torch.int64, device="cuda")
    cap = 400 * nT
    indices = torch.full((cap,), -1, dtype=torch.int32, device="cuda")
    nnz = ctypes.c_int64(-1)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    _lib.call("emg_csr_pattern_noalloc", nT, N, ctypes.c_void_p(t2f.data_ptr()), ctypes.c_void_p(indptr.data_ptr()),
              ctypes.c_void_p(indices.data_ptr()), cap, ctypes.byref(nnz), stream)
    return indptr.cpu().numpy(), indices[: nnz.value].cpu().numpy(), nnz.value


def test_noalloc_pattern_matches_plan_twice_in_a_row(torch_cuda):
    torch = torch_cuda
    from emerge_gb300.assembly import AssemblyPlan
    from emerge_gb300.mesh import Nedelec2Basis, unit_cube
    fields = [Nedelec2Basis(unit_cube(7, jitter=0.15, seed=2)), Nedelec2Basis(unit_cube(4, jitter=0.1, seed=5))]
    for field in fields:                       # second call reuses the scratch left by the first
        ip, ix, nnz = _noalloc_pattern(torch, field)
        plan = AssemblyPlan(field)
        ref_ip, ref_ix = plan.indptr.cpu().numpy(), plan.indices[: plan.nnz].cpu().numpy()
        assert nnz == plan.nnz
        assert np.array_equal(ip, ref_ip)
        assert np.array_equal(ix, ref_ix)


def test_noalloc_rejects_sizes_beyond_its_scratch(torch_cuda):
    torch = torch_cuda
    from emerge_gb300._lib import EmgError
    from emerge_gb300.mesh import Nedelec2Basis, unit_cube
    field = Nedelec2Basis(unit_cube(12))       # 10368 tets > 8192
    with pytest.raises(EmgError, match="too large"):
        _noalloc_pattern(torch, field)
