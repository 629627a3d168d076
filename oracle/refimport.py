"""Test infrastructure only: import the reference package (albert-hzbn/LResDFT `lrft`)
from its source tree together with the C++ extension that `oracle/build_ref.sh`
compiled into `oracle/_ref/`.

The reference imports its extension with `from . import _lrft_cpp`
(lrft/lcao3d.py:307,347); the reference tree is read-only, so the compiled module
is registered under that name in `sys.modules` before the first use.  Only the
golden-vector generator and the optional reference-comparison tests call this;
it needs the reference tree, which exists only in the build container.
"""
from __future__ import annotations

import glob
import importlib.util
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
def reference_root():
    """The reference source tree: the LRES_REFERENCE_ROOT environment variable (no default)."""
    return os.environ.get("LRES_REFERENCE_ROOT")


def available(root=None) -> bool:
    root = root or reference_root()
    return bool(root) and os.path.isfile(os.path.join(root, "lrft", "lcao3d.py"))


def load(root=None, need_cpp: bool = True):
    """Return the reference modules (three_d, lcao3d); registers lrft._lrft_cpp.  The tree is
    `root`, else LRES_REFERENCE_ROOT."""
    root = root or reference_root()
    if not available(root):
        raise ImportError(f"reference tree not found (root {root!r}; set LRES_REFERENCE_ROOT)")
    if root not in sys.path:
        sys.path.insert(0, root)
    import lrft  # noqa: F401
    if need_cpp and "lrft._lrft_cpp" not in sys.modules:
        so = glob.glob(os.path.join(HERE, "_ref", "_lrft_cpp*.so"))
        if not so:
            raise ImportError("oracle/_ref/_lrft_cpp*.so missing: run sh oracle/build_ref.sh")
        spec = importlib.util.spec_from_file_location("lrft._lrft_cpp", so[0])
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        sys.modules["lrft._lrft_cpp"] = mod
        lrft._lrft_cpp = mod
    from lrft import lcao3d, three_d
    return three_d, lcao3d
