"""The C ABI library builds, loads and exports every symbol include/qtgpu.h
declares; argument validation works without touching a GPU (CPU)."""
import ctypes
import os
import re

import pytest

from qutree_gb300 import qtgpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    src = open(os.path.join(ROOT, "include", "qtgpu.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|void|const char\*|int64_t)\s+\**(qt_\w+)\s*\(", src, re.M)))


def test_library_exports_header_symbols():
    L = qtgpu.load()
    names = header_symbols()
    assert len(names) >= 25
    for name in names:
        assert hasattr(L, name), name
    assert sorted(qtgpu.exported_symbols()) == names


def test_null_arguments_are_rejected():
    L = qtgpu.load()
    assert L.qt_ctx_create(None, 0) == 1  # QT_ERR_ARG
    assert b"null" in L.qt_last_error(None)
    # calls on a null context return QT_ERR_ARG instead of crashing
    assert L.qt_sync(None) == 1
    assert L.qt_derivative(None, 1.0, 0.0) == 1
    assert L.qt_psi_size(None) == -1


def test_no_device_is_an_error_not_a_fallback():
    # Without a GPU the context cannot be created; nothing runs on the CPU.
    L = qtgpu.load()
    h = ctypes.c_void_p()
    rc = L.qt_ctx_create(ctypes.byref(h), 0)
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = None
    if has_gpu:
        pytest.skip("a GPU is present")
    assert rc != 0 and not h.value
