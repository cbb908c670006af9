"""The C-ABI library loads without a GPU and exports every symbol include/*.h declares."""
import glob
import os
import re
import subprocess

import pytest

from conftest import ROOT


def _declared():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names.update(re.findall(r"\b(emg_\w+)\s*\(", src))
    return sorted(names)


@pytest.fixture(scope="module")
def libpath():
    from emerge_gb300 import _build
    return _build.build()


def test_header_declares_entry_points():
    names = _declared()
    for n in ("emg_plan_create", "emg_assemble_tet", "emg_assemble_tet_host", "emg_plan_destroy", "emg_last_error"):
        assert n in names


def test_library_exports_all_declared_symbols(libpath):
    out = subprocess.run(["nm", "-D", "--defined-only", libpath], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\bT\s+(emg_\w+)", out))
    missing = [n for n in _declared() if n not in exported]
    assert not missing, missing


def test_library_loads_and_binds(libpath):
    from emerge_gb300 import _lib
    lib = _lib.load(libpath)
    for n in _declared():
        assert hasattr(lib, n)
        assert n in _lib.SIGNATURES, f"{n} has no ctypes signature"
    assert lib.emg_version().startswith(b"emerge_gb300")


def test_argument_errors_are_reported_without_gpu(libpath):
    """Argument validation runs before any CUDA call and reports through emg_last_error."""
    import ctypes
    from emerge_gb300 import _lib
    lib = _lib.load(libpath)
    plan = ctypes.c_void_p()
    rc = lib.emg_plan_create(1, 1, 1, 1, 5, None, None, None, None, None, None, None, None, ctypes.byref(plan))
    assert rc == 1
    assert b"n_field" in lib.emg_last_error()
