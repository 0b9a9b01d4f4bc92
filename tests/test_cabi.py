"""The C-ABI library loads and exports every function include/qt_rgf.h declares.

Runs without a GPU: no compute entry point is called.
"""
import os
import re

from quantum_transport_gb300 import _lib
from quantum_transport_gb300.build import build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    src = open(os.path.join(ROOT, "include", "qt_rgf.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(qt_[a-z0-9_]+)\s*\(", src)))


def test_header_lists_match_binding():
    assert header_functions() == sorted(_lib.EXPORTS)


def test_library_exports_all_symbols():
    build()
    lib = _lib.load()
    for name in header_functions():
        assert hasattr(lib, name), name
    assert lib.qt_version().decode().startswith("qtgpu")


def test_ctx_create_without_gpu_fails_cleanly():
    import ctypes
    import torch
    if torch.cuda.is_available():
        return
    lib = _lib.load()
    h = ctypes.c_void_p()
    rc = lib.qt_ctx_create(ctypes.byref(h), 0)
    assert rc == _lib.QT_ERR_CUDA
    assert lib.qt_last_error()
