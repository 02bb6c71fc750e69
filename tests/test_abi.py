"""
The C ABI library builds for sm_103a without a GPU, loads, and exports every
function that include/*.h declares (no compute calls: this runs on CPU).
"""

import ctypes
import glob
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for header in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(header).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names.update(re.findall(r"\b(hg_\w+)\s*\(", text))
    return sorted(names)


def test_library_exports_declared_symbols():
    from harmonica_gb300 import _native

    _native.build()
    handle = ctypes.CDLL(_native.LIB_PATH)
    names = declared_functions()
    assert "hg_prism_forward" in names and "hg_layer_forward" in names
    missing = [n for n in names if not hasattr(handle, n)]
    assert not missing, f"symbols declared but not exported: {missing}"
    # every declared symbol has a ctypes prototype in the Python binding
    assert set(names) <= set(_native.PROTOTYPES), set(names) - set(_native.PROTOTYPES)


def test_version_and_error_without_gpu():
    from harmonica_gb300 import _native

    lib = _native.lib()
    assert lib.hg_version() >= 100
    # argument validation happens before any CUDA call
    size = ctypes.c_size_t(0)
    assert lib.hg_prism_forward_workspace(-1, 10, 1, ctypes.byref(size)) < 0
    assert b"bad sizes" in lib.hg_last_error()
    assert lib.hg_prism_forward_workspace(10, 10, 0, ctypes.byref(size)) < 0
    assert lib.hg_prism_forward_workspace(2500, 10000, 1 << 3, ctypes.byref(size)) == 0
