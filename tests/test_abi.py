"""CPU checks of the C ABI: the library builds, loads, and exports exactly the
symbols include/covertree_cuda.h declares (no compute calls without a GPU)."""
import re
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _declared():
    text = (ROOT / "include" / "covertree_cuda.h").read_text()
    return sorted(set(re.findall(r"CT_API\s+[\w\s\*]*?\b(ct_\w+)\s*\(", text)))


def test_header_declares_entry_points():
    names = _declared()
    assert "ct_build_residual" in names and "ct_knn_residual" in names and "ct_free" in names


def test_library_exports_every_declared_symbol():
    from covertreex_gb300 import _build, _lib

    path = _build.build_library()
    out = subprocess.run(["nm", "-D", "--defined-only", str(path)], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\bT (ct_\w+)", out))
    declared = set(_declared())
    assert declared <= exported, declared - exported
    assert exported <= declared, exported - declared
    assert set(_lib.EXPORTED_SYMBOLS) == declared


def test_library_loads_and_reports_version():
    from covertreex_gb300 import _lib

    L = _lib.load()
    assert L.ct_version() >= 10000
    assert L.ct_last_error() == b""


def test_null_arguments_are_rejected_without_gpu_work():
    import ctypes

    from covertreex_gb300 import _lib

    L = _lib.load()
    rc = L.ct_build_residual(None, None, None, 10, 16, 3, 1.0, None, 0, 0, 512, 1, 0, 0, None, None)
    assert rc == _lib.CT_ERR_ARG
    assert b"out is NULL" in L.ct_last_error()
    h = ctypes.c_void_p()
    rc = L.ct_build_residual(None, None, None, 10, 17, 3, 1.0, None, 0, 0, 512, 1, 0, 0, None, ctypes.byref(h))
    assert rc == _lib.CT_ERR_UNSUPPORTED
    rc = L.ct_knn_residual(None, None, 1, 5, 0, 0, None, None, None, None)
    assert rc == _lib.CT_ERR_ARG
