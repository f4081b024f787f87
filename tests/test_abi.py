"""CPU checks of the C ABI: libdmsc.so builds for sm_103a, loads, and exports
every entry point declared in include/dmsc.h (no compute calls without a GPU)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "dmsc.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(dmsc_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_entry_points():
    names = declared_functions()
    assert "dmsc_init" in names and "dmsc_dataset_work" in names
    assert len(names) >= 14


def test_library_exports_every_declared_symbol():
    from mscomplex_gb300 import build
    path = build.build()
    lib = ctypes.CDLL(path)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, f"symbols declared in include/dmsc.h but not exported: {missing}"


def test_python_binding_covers_header():
    from mscomplex_gb300 import _native
    missing = [n for n in declared_functions() if n not in _native.SIGNATURES]
    assert not missing, f"entry points without a ctypes signature: {missing}"


def test_errors_without_gpu_are_reported():
    import torch
    if torch.cuda.is_available():
        pytest.skip("GPU present; covered by the gpu tests")
    from mscomplex_gb300 import _native
    lib = _native.load()
    h = ctypes.c_void_p()
    rc = lib.dmsc_init(0, ctypes.byref(h))
    assert rc != 0
    assert lib.dmsc_last_error()
