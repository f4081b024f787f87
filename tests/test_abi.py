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


NULL_CALLS = r'''
import ctypes, re, sys
from mscomplex_gb300 import build
lib = ctypes.CDLL(build.build())
lib.dmsc_last_error.restype = ctypes.c_char_p
for spec in sys.argv[1:]:
    name, nargs = spec.split(":")
    f = getattr(lib, name)
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p] * int(nargs)
    print(name, flush=True)  # the last name printed is the one that crashed, if any
    rc = f(*([None] * int(nargs)))
    msg = lib.dmsc_last_error().decode()
    print(name, rc, msg, flush=True)
'''


def test_null_arguments_are_errors_not_crashes():
    """Every entry point, given null handles and pointers (and zeros), returns
    an error with a message -- the reference's exceptions become statuses --
    instead of dereferencing them.  Needs no GPU: the checks precede any CUDA call."""
    import subprocess
    import sys
    src = open(os.path.join(ROOT, "include", "dmsc.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    specs = []
    for name, args in re.findall(r"\bint\s+(dmsc_[a-z0-9_]+)\s*\(([^)]*)\)", src):
        n = 0 if args.strip() in ("", "void") else args.count(",") + 1
        if n:
            specs.append(f"{name}:{n}")
    assert len(specs) >= 40
    r = subprocess.run([sys.executable, "-c", NULL_CALLS, *specs], capture_output=True, text=True, timeout=300,
                       cwd=ROOT)
    lines = [l.split(" ", 2) for l in r.stdout.splitlines() if l.count(" ") >= 2]
    assert r.returncode == 0, f"crashed after {r.stdout.splitlines()[-1:]}: {r.stderr[-500:]}"
    assert len(lines) == len(specs)
    for name, rc, msg in lines:
        assert int(rc) != 0 and msg.strip(), f"{name} accepted null arguments (rc {rc}, message {msg!r})"
