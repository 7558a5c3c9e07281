"""The C-ABI library builds for sm_103a and exports every symbol declared in
include/pnfam_gpu.h (no GPU needed: nothing is called)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    txt = open(os.path.join(ROOT, "include", "pnfam_gpu.h")).read()
    return sorted(set(re.findall(r"\b(pnfam_gpu_\w+)\s*\(", txt)))


def test_library_exports_header_symbols():
    from pynfam_gb300 import build, _lib
    path = build.build()
    lib = ctypes.CDLL(path)
    syms = declared_symbols()
    assert len(syms) >= 8
    for s in syms:
        assert hasattr(lib, s), s
    assert set(_lib.EXPORTS) <= set(syms)


def test_error_message_without_context():
    from pynfam_gb300 import _lib
    lib = _lib.load()
    rc = lib.pnfam_gpu_set_operator(None, 1, None, None, 0, None)
    assert rc == 1 and b"bad argument" in lib.pnfam_gpu_last_error()
