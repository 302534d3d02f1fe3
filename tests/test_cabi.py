"""The C-ABI library builds, loads, and exports every symbol include/fvm_gpu.h declares
(no compute calls: there is no GPU here)."""
import ctypes
import re
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "fvm_gpu.h"


def declared_symbols():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\bint\s+(fvm_\w+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    from fvmgpu import _build, _lib

    path = _build.build()
    lib = ctypes.CDLL(str(path))
    syms = declared_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(lib, s), s
    assert set(syms) == set(_lib.SIGNATURES), "ctypes signatures must mirror the header"
    out = subprocess.run(["nm", "-D", "--defined-only", str(path)], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (fvm_\w+)", out))
    assert set(syms) <= exported


def test_version_device_count_and_last_error():
    from fvmgpu import _lib

    lib = _lib.load()
    assert lib.fvm_version() >= 10000
    n = ctypes.c_int(-1)
    assert lib.fvm_device_count(ctypes.byref(n)) == 0 and n.value >= 0
    buf = ctypes.create_string_buffer(64)
    assert lib.fvm_last_error(buf, len(buf)) == 0
    assert lib.fvm_last_error(None, 0) == _lib.FVM_ERR_INVALID_ARGUMENT


def test_null_arguments_return_status_not_crash():
    from fvmgpu import _lib

    lib = _lib.load()
    assert lib.fvm_mesh_create(None, 0, None, 0, None, None, 0, 0, 0, None) == _lib.FVM_ERR_INVALID_ARGUMENT
    assert lib.fvm_rhs(None, None, None, 0.0, 0, None) == _lib.FVM_ERR_INVALID_ARGUMENT
    assert lib.fvm_problem_create(None, None, None) == _lib.FVM_ERR_INVALID_ARGUMENT
    assert lib.fvm_template_create(None, 0, None) == _lib.FVM_ERR_INVALID_ARGUMENT
    assert "NULL" in _lib.last_error() or _lib.last_error()


def test_no_cpu_fallback_without_gpu():
    """The product path refuses to run without a device (there is no CPU fallback)."""
    from fvmgpu import _lib

    if _lib.device_count() > 0:
        pytest.skip("a GPU is present")
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        _lib.require_gpu()
