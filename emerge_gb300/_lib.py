"""ctypes binding of the C ABI in include/emerge_gb300.h.

The shared library is built in-tree (``emerge_gb300/libemerge_gb300.so``, see
``_build.py``).  There is no CPU fallback: if the library is missing or a call
fails, an exception is raised.
"""
from __future__ import annotations

import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libemerge_gb300.so")

c_i64 = ctypes.c_int64
c_i32p = ctypes.POINTER(ctypes.c_int32)
c_i64p = ctypes.POINTER(ctypes.c_int64)
c_f64p = ctypes.POINTER(ctypes.c_double)
c_vp = ctypes.c_void_p

# name -> (restype, argtypes); mirrors include/emerge_gb300.h
SIGNATURES = {
    "emg_last_error": (ctypes.c_char_p, []),
    "emg_version": (ctypes.c_char_p, []),
    "emg_plan_create": (ctypes.c_int, [c_i64, c_i64, c_i64, c_i64, c_i64, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp,
                                       c_vp, ctypes.POINTER(c_vp)]),
    "emg_plan_nnz": (c_i64, [c_vp]),
    "emg_plan_pattern": (ctypes.c_int, [c_vp, c_vp, c_vp, c_vp]),
    "emg_assemble_tet": (ctypes.c_int, [c_vp, c_vp, c_vp, c_vp, c_vp, c_vp]),
    "emg_assemble_tet_host": (ctypes.c_int, [c_vp, c_vp, c_vp, c_vp, c_vp, c_vp]),
    "emg_assemble_tet_tensor": (ctypes.c_int, [c_vp, c_vp, c_vp, c_vp, c_vp, c_vp]),
    "emg_topology_create": (ctypes.c_int, [c_i64, c_i64, c_vp, c_vp, c_vp]),
    "emg_topology_sizes": (ctypes.c_int, [c_vp, c_vp, c_vp]),
    "emg_topology_get": (ctypes.c_int, [c_vp] * 9),
    "emg_topology_destroy": (None, [c_vp]),
    "emg_edge_lengths": (ctypes.c_int, [c_i64, c_vp, c_i64, c_vp, c_vp, c_vp]),
    "emg_field_weights": (ctypes.c_int, [c_i64, c_vp, c_vp, c_i64, c_vp, c_i64, c_vp, c_i64, c_vp, c_i64, c_vp, c_vp,
                                         c_i64, c_vp, c_vp, c_vp, c_vp]),
    "emg_port_element_matrices": (ctypes.c_int, [c_i64, c_vp, c_vp, c_vp, c_vp, ctypes.c_double, ctypes.c_int, c_vp,
                                                 c_vp, c_vp]),
    "emg_stratton_chu": (ctypes.c_int, [c_i64, c_vp, c_vp, c_vp, c_vp, c_i64, c_vp, c_vp, ctypes.c_float, c_vp,
                                        c_vp, c_vp]),
    "emg_assemble_tet_tensor_host": (ctypes.c_int, [c_vp, c_vp, c_vp, c_vp, c_vp, c_vp]),
    "emg_plan_destroy": (None, [c_vp]),
    "emg_tri_robin_force": (ctypes.c_int, [c_i64, c_vp, c_vp, c_vp, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                           c_vp, c_vp, c_vp]),
    "emg_tri_robin_abc": (ctypes.c_int, [c_i64, c_vp, c_vp, ctypes.c_double, ctypes.c_double, c_vp, c_vp]),
    "emg_csr_positions": (ctypes.c_int, [c_i64, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp]),
    "emg_segment_add": (ctypes.c_int, [c_i64, c_vp, c_vp, c_vp, c_vp, ctypes.c_double, ctypes.c_double, c_vp, c_vp]),
    "emg_combine": (ctypes.c_int, [c_i64, c_vp, c_vp, ctypes.c_double, c_vp, c_vp]),
    "emg_matinv": (ctypes.c_int, [c_i64, ctypes.c_int, c_vp, c_vp, c_vp]),
    "emg_port_interp": (ctypes.c_int, [c_i64, c_vp, c_i64, c_vp, c_i64, c_vp, c_vp, c_vp, c_vp, ctypes.c_double,
                                       ctypes.c_int, c_vp, c_vp]),
    "emg_rplan_create": (ctypes.c_int, [c_i64, c_vp, c_vp, c_i64, c_i64, c_vp, c_vp, ctypes.POINTER(c_vp)]),
    "emg_rplan_n": (c_i64, [c_vp]),
    "emg_rplan_nnz": (c_i64, [c_vp]),
    "emg_rplan_levels": (c_i64, [c_vp]),
    "emg_rplan_destroy": (None, [c_vp]),
    "emg_rplan_form": (ctypes.c_int, [c_vp, c_i64, c_vp, c_vp, c_vp, c_i64, c_vp, c_vp, c_vp, c_vp]),
    "emg_ilu0": (ctypes.c_int, [c_vp, c_i64, c_vp, c_vp]),
    "emg_ilu_apply": (ctypes.c_int, [c_vp, c_i64, c_vp, c_i64, c_vp, c_vp, c_vp]),
    "emg_spmv": (ctypes.c_int, [c_vp, c_i64, c_vp, c_i64, c_vp, c_vp, c_vp, c_vp, c_vp]),
    "emg_rplan_gather": (ctypes.c_int, [c_vp, c_i64, c_vp, c_vp, c_vp]),
    "emg_rplan_scatter": (ctypes.c_int, [c_vp, c_i64, c_vp, c_vp, c_vp]),
    "emg_gmres": (ctypes.c_int, [c_vp, c_i64, c_vp, c_i64, c_vp, c_vp, c_vp, c_vp, ctypes.c_int, ctypes.c_int,
                                 ctypes.c_double, c_vp, c_vp, c_vp]),
    "emg_rplan_pattern": (ctypes.c_int, [c_vp, c_vp, c_vp]),
    "emg_spmv_family": (ctypes.c_int, [c_vp, c_i64, ctypes.c_int, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp]),
    "emg_gmres_slab_family": (ctypes.c_int, [c_vp, c_vp, c_i64, ctypes.c_int, c_vp, c_vp, c_vp, c_vp, c_vp,
                                             ctypes.c_int, ctypes.c_int, ctypes.c_double, c_vp, c_vp, c_vp]),
    "emg_gmres_slab_mixed": (ctypes.c_int, [c_vp, c_vp, c_i64, c_vp, c_i64, c_vp, c_vp, c_vp, c_vp, ctypes.c_int,
                                            ctypes.c_int, ctypes.c_double, ctypes.c_double, c_vp, c_vp, c_vp, c_vp]),
    "emg_tc_gemm_tf32": (ctypes.c_int, [c_i64, c_i64, c_i64, c_vp, c_i64, c_vp, c_i64, c_vp, c_i64, c_vp, c_vp]),
    "emg_slab_set_tensor_cores": (ctypes.c_int, [c_vp, ctypes.c_int]),
    "emg_slab_set_factor_tensor_cores": (ctypes.c_int, [c_vp, ctypes.c_int]),
    "emg_slab_set_wide_group": (ctypes.c_int, [c_vp, ctypes.c_int]),
    "emg_slab_set_max_splits": (ctypes.c_int, [c_vp, ctypes.c_int]),
    "emg_field_interp": (ctypes.c_int, [c_i64, c_vp, c_i64, c_vp, c_i64, c_vp, c_i64, c_vp, c_i64, c_vp, c_vp, c_vp,
                                        c_i64, c_vp, c_vp, c_vp]),
    "emg_slab_create": (ctypes.c_int, [c_vp, c_i64, c_vp, c_vp, c_vp, ctypes.POINTER(c_vp)]),
    "emg_slab_destroy": (None, [c_vp]),
    "emg_slab_info": (ctypes.c_int, [c_vp, c_vp]),
    "emg_slab_levels": (ctypes.c_int, [c_vp, c_vp, c_vp]),
    "emg_slab_factor": (ctypes.c_int, [c_vp, ctypes.c_int, c_i64, c_vp, c_i64, c_vp, ctypes.c_int, c_vp]),
    "emg_slab_apply": (ctypes.c_int, [c_vp, c_i64, c_vp, c_vp, c_vp, c_vp]),
    "emg_gmres_slab": (ctypes.c_int, [c_vp, c_vp, c_i64, c_vp, c_i64, c_vp, c_vp, c_vp, c_vp, ctypes.c_int,
                                      ctypes.c_int, ctypes.c_double, c_vp, c_vp, c_vp]),
    "emg_mlp_create": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                      ctypes.c_uint64, ctypes.POINTER(c_vp)]),
    "emg_mlp_nparam": (c_i64, [c_vp]),
    "emg_mlp_get_params": (ctypes.c_int, [c_vp, c_vp]),
    "emg_mlp_set_params": (ctypes.c_int, [c_vp, c_vp]),
    "emg_mlp_forward": (ctypes.c_int, [c_vp, ctypes.c_int, c_vp, c_vp, c_vp]),
    "emg_mlp_train_step": (ctypes.c_int, [c_vp, ctypes.c_int, c_vp, c_vp, ctypes.c_float, c_vp, c_vp, c_vp]),
    "emg_mlp_destroy": (None, [c_vp]),
    "emg_csr_pattern_noalloc": (ctypes.c_int, [c_i64, c_i64, c_vp, c_vp, c_vp, c_i64, c_i64p, c_vp]),
}


class EmgError(RuntimeError):
    """A C-ABI call returned a nonzero status."""

    def __init__(self, fn: str, code: int, msg: str):
        super().__init__(f"{fn} failed (status {code}): {msg}")
        self.code = code


_lib = None


def load(path: str = LIB_PATH):
    """Load (once) and return the shared library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"CUDA library not built: {path} is missing (run __graft_entry__.build() or "
                           f"python -m emerge_gb300._build)")
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(fn: str, code: int) -> None:
    if code != 0:
        msg = load().emg_last_error()
        raise EmgError(fn, code, msg.decode() if msg else "")


def call(fn: str, *args):
    """Call ``fn`` and raise EmgError on a nonzero status."""
    code = getattr(load(), fn)(*args)
    check(fn, code)
    return code
