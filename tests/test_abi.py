"""The C-ABI library loads and exports every entry point of include/ocl_gb300.h
(no compute: runs without a GPU)."""
import ctypes
import os
import re

from opencamlib_gb300 import _native

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    src = open(os.path.join(ROOT, "include", "ocl_gb300.h")).read()
    return sorted(set(re.findall(r"\b(ocl_gb300_[a-z_]+)\s*\(", src)))


def test_header_and_binding_agree():
    assert _declared() == sorted(_native.EXPORTS)


def test_library_exports_every_symbol():
    lib = ctypes.CDLL(_native.LIB_PATH)
    for name in _declared():
        assert hasattr(lib, name), name
