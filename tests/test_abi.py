"""The C-ABI library builds for sm_103a, loads on the CPU and exports every entry
point declared in include/lres_gb300.h (no compute calls without a GPU)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    src = open(os.path.join(ROOT, "include", "lres_gb300.h")).read()
    return sorted(set(re.findall(r"\b(lres_[a-z_0-9]+)\s*\(", src)))


def test_header_declarations_are_bound():
    from lresdft_gb300 import _lib
    assert set(declared()) == set(_lib.EXPORTS)


def test_library_exports_every_declared_symbol():
    from lresdft_gb300 import _lib
    lib = ctypes.CDLL(_lib.LIB_PATH)
    for name in declared():
        assert hasattr(lib, name), name
    assert _lib.lib.lres_version().decode().startswith("lres_gb300")


def test_errors_are_reported_not_raised():
    from lresdft_gb300 import _lib
    rc = _lib.lib.lres_ctx_create(None, None, 0, 64, None)
    assert rc == -22
    assert b"null" in _lib.lib.lres_last_error()
    with pytest.raises(_lib.LResError):
        _lib.check(rc)
