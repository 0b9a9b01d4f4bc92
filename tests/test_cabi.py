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


def header_constants():
    """Enumerators and #define values of include/qt_rgf.h."""
    src = open(os.path.join(ROOT, "include", "qt_rgf.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    vals = {m[0]: int(m[1]) for m in re.findall(r"#define\s+(QT_[A-Z0-9_]+)\s+(\d+)u?\b", src)}
    vals.update({m[0]: int(m[1]) for m in re.findall(r"\b(QT_[A-Z0-9_]+)\s*=\s*(\d+)", src)})
    return vals


def test_header_constants_match_binding():
    consts = header_constants()
    names = [n for n in dir(_lib) if n.startswith("QT_") and isinstance(getattr(_lib, n), int)]
    assert names
    for name in names:
        assert consts.get(name) == getattr(_lib, name), name
    for name in ("QT_PREC_FP64", "QT_PREC_MIXED", "QT_PREC_MIXED_FP64", "QT_ERR_POINTS",
                 "QT_FLAG_CAROLI", "QT_QUIRK_GLP_ZERO"):
        assert name in names, name
