"""
The C ABI library builds for sm_103a without a GPU, loads, and exports every
function that include/*.h declares (no compute calls: this runs on CPU).
"""

import ctypes
import glob
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions(header_name="harmonica_gb300.h"):
    names = set()
    for header in glob.glob(os.path.join(ROOT, "include", header_name)):
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


def test_bench_library_is_separate_and_exports_its_header():
    """The benchmark probes (include/harmonica_gb300_bench.h) live in their
    own library, not in the product library."""
    from harmonica_gb300 import _native

    _native.build()
    product = ctypes.CDLL(_native.LIB_PATH)
    bench = ctypes.CDLL(_native.BENCH_LIB_PATH)
    names = declared_functions("harmonica_gb300_bench.h")
    assert names
    for n in names:
        assert hasattr(bench, n), n
        assert not hasattr(product, n), n


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


def test_header_compiles_and_links_as_c(tmp_path):
    """include/harmonica_gb300.h is a C header: a C99 program that includes
    it builds with -Wall -Wextra -pedantic -Werror, links against the
    library and passes its GPU-free checks (tests/native/abi_consumer.c)."""
    import shutil
    import subprocess

    import pytest

    from harmonica_gb300 import _native

    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("gcc not available")
    _native.build()
    exe = str(tmp_path / "abi_consumer")
    subprocess.run(
        [gcc, "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror",
         "-I", os.path.join(ROOT, "include"),
         os.path.join(ROOT, "tests", "native", "abi_consumer.c"),
         "-L", _native.BUILD_DIR, "-lharmonica_gb300",
         "-Wl,-rpath," + _native.BUILD_DIR, "-o", exe],
        check=True, capture_output=True, text=True)
    run = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert run.returncode == 0, run.stderr
    assert "all checks passed" in run.stdout


def test_tesseroid_and_eqs_validation_without_gpu():
    """Argument checks of the tesseroid and equivalent-source entry points
    (they return before any CUDA call)."""
    from harmonica_gb300 import _native

    lib = _native.lib()
    size = ctypes.c_size_t(0)
    assert lib.hg_tesseroid_forward_workspace(-1, 10, ctypes.byref(size)) < 0
    assert b"bad sizes" in lib.hg_last_error()
    assert lib.hg_tesseroid_forward_workspace(100, 1000, ctypes.byref(size)) == 0
    assert size.value >= 52 * 1000 * 8  # the prepared tesseroid records
    args = [None, None, None, 1, None, None, 0, 1]
    # radial, stack size, max discretizations, nodes, weights, out, status,
    # workspace, workspace bytes, stream
    tail = [0, 100, 0, None, None, None, None, None, 0, None]
    # field other than potential (0) or g_z (3)
    assert lib.hg_tesseroid_forward(*args, 5, *tail) < 0
    assert b"tesseroid field" in lib.hg_last_error()
    # stack larger than the kernels' 100 entries
    tail_big_stack = [0, 101, 0, None, None, None, None, None, 0, None]
    assert lib.hg_tesseroid_forward(*args, 3, *tail_big_stack) < 0
    assert b"stack size above 100" in lib.hg_last_error()
    # null pointers with work to do
    assert lib.hg_tesseroid_forward(*args, 3, *tail) < 0
    assert b"null pointer" in lib.hg_last_error()
    assert lib.hg_tesseroid_inside(None, None, None, 1, None, 1, None, 0, None, None) < 0
    assert b"null pointer" in lib.hg_last_error()
    assert lib.hg_eqs_jacobian(None, None, None, -1, None, None, None, 1, 0, None, None) < 0
    assert b"bad sizes" in lib.hg_last_error()
    assert lib.hg_eqs_jacobian(None, None, None, 2, None, None, None, 3, 0, None, None) < 0
    assert b"null pointer" in lib.hg_last_error()
    assert lib.hg_eqs_predict(None, None, None, 2, None, None, None, None, 3, 0, None, None, 0,
                              None) < 0
    assert b"null pointer" in lib.hg_last_error()


def test_noalloc_validation_without_gpu():
    """hg_prism_forward_noalloc checks its arguments before any CUDA call:
    negative sizes, a bad field mask, a prism stride below the prism count
    and null pointers with work to do are rejected with a message."""
    from harmonica_gb300 import _native

    lib = _native.lib()
    f = lib.hg_prism_forward_noalloc
    assert f(None, None, None, -1, None, 10, 10, 1 << 3, None, None, None) < 0
    assert b"bad sizes" in lib.hg_last_error()
    assert f(None, None, None, 4, None, 10, 10, 0, None, None, None) < 0
    assert b"field mask" in lib.hg_last_error()
    assert f(None, None, None, 4, None, 10, 10, 1 << 10, None, None, None) < 0
    assert f(None, None, None, 4, None, 5, 10, 1 << 3, None, None, None) < 0
    assert b"bad sizes" in lib.hg_last_error()
    assert f(None, None, None, 4, None, 10, 10, 1 << 3, None, None, None) < 0
    assert b"null pointer" in lib.hg_last_error()
    assert lib.hg_prism_forward_noalloc(
        ctypes.c_void_p(8), ctypes.c_void_p(8), ctypes.c_void_p(8), 4, None, 10, 10, 1 << 3,
        ctypes.c_void_p(8), None, None) < 0
    assert b"null prisms pointer" in lib.hg_last_error()


_PROBE = r"""
import ctypes, json, sys
sys.path.insert(0, sys.argv[1])
from harmonica_gb300 import _native
lib = _native.lib()
report = {}
for name, (res, args) in _native.PROTOTYPES.items():
    if not args or name == "hg_batch_destroy":
        continue
    for mode in ("negative sizes", "null pointers"):
        vals = []
        for a in args:
            if a in (ctypes.c_int64, ctypes.c_int32, ctypes.c_int):
                vals.append(-1 if mode == "negative sizes" else 3)
            elif a is ctypes.c_uint32:
                vals.append(1 << 3)
            elif a is ctypes.c_size_t:
                vals.append(0)
            elif a is ctypes.c_double:
                vals.append(0.0)
            else:
                vals.append(None)
        rc = getattr(lib, name)(*vals)
        report[name + ": " + mode] = [rc, lib.hg_last_error().decode()]
print(json.dumps(report))
"""


def test_every_entry_point_rejects_bad_arguments_before_cuda():
    """Every function of the C ABI, called with negative sizes or with null
    pointers, returns HG_ERR_INVALID with a message and touches neither
    memory nor the GPU (run in a child process, so a crash fails the test
    instead of the test run)."""
    import json
    import subprocess
    import sys

    from harmonica_gb300 import _native

    _native.build()
    run = subprocess.run([sys.executable, "-c", _PROBE, ROOT], capture_output=True, text=True,
                         timeout=300)
    assert run.returncode == 0, run.stderr[-2000:]
    report = json.loads(run.stdout.strip().splitlines()[-1])
    declared = set(declared_functions()) - {"hg_version", "hg_last_error", "hg_batch_destroy"}
    assert {k.split(":")[0] for k in report} == declared
    bad = {k: v for k, v in report.items() if v[0] != -1 or not v[1]}
    assert not bad, bad


_LOCK_CHILD = r"""
import sys, time
sys.path.insert(0, sys.argv[1])
from harmonica_gb300 import _native

def fake_compile(verbose):
    start = time.time()
    time.sleep(0.5)
    with open(sys.argv[2], "a") as log:
        log.write(f"{start} {time.time()}\n")

_native._compile_and_link = fake_compile
_native.build(force=True)
"""


def test_concurrent_builds_are_serialised(tmp_path):
    """Two processes building at once take turns on the build lock (the
    compile step is replaced by a half-second stub in the children)."""
    import subprocess
    import sys

    log = tmp_path / "intervals.txt"
    procs = [subprocess.Popen([sys.executable, "-c", _LOCK_CHILD, ROOT, str(log)])
             for _ in range(2)]
    assert all(p.wait(timeout=120) == 0 for p in procs)
    (a0, a1), (b0, b1) = sorted(tuple(map(float, line.split()))
                                for line in log.read_text().splitlines())
    assert a1 <= b0  # the second build started after the first one ended
