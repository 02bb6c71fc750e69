"""
Build and load the native library ``libharmonica_gb300.so`` (CUDA kernels for
sm_103a plus the C ABI declared in ``include/harmonica_gb300.h``).

The library is built in-tree (``harmonica_gb300/_build/``) by :func:`build`
and loaded with :mod:`ctypes`.  There is no fallback: if the library is
missing, :func:`lib` raises, so a GPU run can never silently compute on the
CPU.
"""

import contextlib
import ctypes
import os
import shutil
import subprocess
import threading

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
REPO_DIR = os.path.dirname(PKG_DIR)
CSRC_DIR = os.path.join(PKG_DIR, "csrc")
BUILD_DIR = os.path.join(PKG_DIR, "_build")
LIB_NAME = "libharmonica_gb300.so"
LIB_PATH = os.path.join(BUILD_DIR, LIB_NAME)
HEADERS = (
    os.path.join(REPO_DIR, "include", "harmonica_gb300.h"),
    os.path.join(REPO_DIR, "include", "harmonica_gb300_bench.h"),
)

#: translation units compiled into the library
SOURCES = (
    "prism_forward.cu", "prism_batch.cu", "prism_batch64.cu", "prism_adjoint.cu",
    "point_forward.cu", "prism_magnetic.cu", "tesseroid_forward.cu",
)
#: the benchmark-support library (include/harmonica_gb300_bench.h), kept out
#: of the product library; it links against the product library
BENCH_SOURCES = ("bench_probe.cu",)
BENCH_LIB_PATH = os.path.join(BUILD_DIR, "libhg_bench.so")

ARCH_FLAGS = ("-gencode", "arch=compute_103a,code=sm_103a")

_lock = threading.Lock()
_lib = None


def nvcc_path():
    cand = shutil.which("nvcc")
    if cand:
        return cand
    default = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(default):
        return default
    raise RuntimeError("nvcc not found: cannot build the harmonica_gb300 CUDA library")


def _sources(names=SOURCES):
    return [os.path.join(CSRC_DIR, s) for s in names]


def _deps():
    deps = _sources(SOURCES + BENCH_SOURCES) + list(HEADERS)
    deps += [
        os.path.join(CSRC_DIR, f) for f in os.listdir(CSRC_DIR) if f.endswith((".cuh", ".h"))
    ]
    return deps


def is_stale():
    if not (os.path.exists(LIB_PATH) and os.path.exists(BENCH_LIB_PATH)):
        return True
    t = min(os.path.getmtime(LIB_PATH), os.path.getmtime(BENCH_LIB_PATH))
    return any(os.path.getmtime(d) > t for d in _deps())


@contextlib.contextmanager
def _build_lock():
    """Exclusive lock across processes (ranks of one job, test workers) on
    the build folder, so that only one of them compiles and links at a time."""
    import fcntl  # noqa: PLC0415

    os.makedirs(BUILD_DIR, exist_ok=True)
    with open(os.path.join(BUILD_DIR, ".build.lock"), "w") as handle:
        fcntl.flock(handle, fcntl.LOCK_EX)
        try:
            yield
        finally:
            fcntl.flock(handle, fcntl.LOCK_UN)


def build(force=False, verbose=False):
    """Compile every CUDA translation unit for sm_103a into one shared library.

    Objects are compiled in parallel, then linked with nvcc (static cudart).
    Concurrent calls from several processes build once: the others wait for
    the lock and find the library up to date (unless ``force``).
    """
    if not force and not is_stale():
        return LIB_PATH
    with _build_lock():
        if not force and not is_stale():  # built by another process meanwhile
            return LIB_PATH
        _compile_and_link(verbose)
    return LIB_PATH


def _compile_and_link(verbose):
    nvcc = nvcc_path()
    common = [
        nvcc, *ARCH_FLAGS, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
        "--expt-relaxed-constexpr", "-I", os.path.join(REPO_DIR, "include"),
    ]
    procs = []
    objs = []
    for src in _sources(SOURCES + BENCH_SOURCES):
        obj = os.path.join(BUILD_DIR, os.path.basename(src) + ".o")
        objs.append(obj)
        cmd = common + ["-c", src, "-o", obj]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    for cmd, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError(
                "nvcc failed:\n" + " ".join(cmd) + "\n" + out.decode(errors="replace")
            )
        if verbose and out:
            print(out.decode(errors="replace"))
    n_product = len(SOURCES)
    _link(nvcc, objs[:n_product], LIB_PATH, [])
    # the bench library resolves the product library's symbols (errors) at
    # load time, found next to it
    _link(nvcc, objs[n_product:], BENCH_LIB_PATH,
          ["-L", BUILD_DIR, "-lharmonica_gb300", "-Xlinker", "-rpath=$ORIGIN"])


def _link(nvcc, objs, path, extra):
    tmp = f"{path}.{os.getpid()}.tmp"
    link = [nvcc, *ARCH_FLAGS, "-shared", "-o", tmp, *objs, *extra]
    res = subprocess.run(link, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if res.returncode != 0:
        raise RuntimeError("nvcc link failed:\n" + res.stdout.decode(errors="replace"))
    os.replace(tmp, path)  # atomic: a loader sees the old or the new library


_c_double_p = ctypes.c_void_p  # device pointers travel as integers


class HgProblemPlan(ctypes.Structure):
    """ctypes mirror of ``hg_problem_plan`` (include/harmonica_gb300.h)."""

    _fields_ = [
        ("obs_e", ctypes.c_void_p),
        ("obs_n", ctypes.c_void_p),
        ("obs_u", ctypes.c_void_p),
        ("n_obs", ctypes.c_int64),
        ("prisms_soa", ctypes.c_void_p),
        ("prism_stride", ctypes.c_int64),
        ("n_prisms", ctypes.c_int64),
        ("chunk", ctypes.c_int64),
        ("n_chunks", ctypes.c_int64),
        ("partials", ctypes.c_void_p),
        ("out", ctypes.c_void_p),
        ("singular_flag", ctypes.c_void_p),
        ("field", ctypes.c_int32),
        ("check_singular", ctypes.c_int32),
    ]


class HgBatchShape(ctypes.Structure):
    """ctypes mirror of ``hg_batch_shape`` (include/harmonica_gb300.h)."""

    _fields_ = [
        ("chunk_prisms", ctypes.c_int64),
        ("points_per_cta", ctypes.c_int32),
        ("n_ctas", ctypes.c_int32),
    ]


class HgProblem(ctypes.Structure):
    """ctypes mirror of ``hg_problem`` (include/harmonica_gb300.h)."""

    _fields_ = [
        ("obs_e", ctypes.c_void_p),
        ("obs_n", ctypes.c_void_p),
        ("obs_u", ctypes.c_void_p),
        ("n_obs", ctypes.c_int64),
        ("prisms_soa", ctypes.c_void_p),
        ("prism_stride", ctypes.c_int64),
        ("n_prisms", ctypes.c_int64),
        ("field", ctypes.c_int32),
        ("check_singular", ctypes.c_int32),
        ("out", ctypes.c_void_p),
        ("singular_flag", ctypes.c_void_p),
    ]

#: ctypes prototypes of every exported symbol (must match include/harmonica_gb300.h)
PROTOTYPES = {
    "hg_version": (ctypes.c_int, []),
    "hg_last_error": (ctypes.c_char_p, []),
    "hg_pack_prisms": (
        ctypes.c_int,
        [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64,
         ctypes.c_void_p],
    ),
    "hg_layer_top_bottom": (
        ctypes.c_int,
        [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double, ctypes.c_int64, ctypes.c_void_p,
         ctypes.c_void_p, ctypes.c_void_p],
    ),
    "hg_prism_forward_workspace": (
        ctypes.c_int,
        [ctypes.c_int64, ctypes.c_int64, ctypes.c_uint32, ctypes.POINTER(ctypes.c_size_t)],
    ),
    "hg_prism_forward": (
        ctypes.c_int,
        [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
         ctypes.c_int64, ctypes.c_int64, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p,
         ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p],
    ),
    "hg_batch_create": (
        ctypes.c_int,
        [ctypes.POINTER(HgProblem), ctypes.c_int64, ctypes.c_int64, ctypes.c_int32,
         ctypes.POINTER(ctypes.c_void_p)],
    ),
    "hg_batch_create_shaped": (
        ctypes.c_int,
        [ctypes.POINTER(HgProblem), ctypes.c_int64, ctypes.POINTER(HgBatchShape),
         ctypes.POINTER(ctypes.c_void_p)],
    ),
    "hg_batch_workspace": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_size_t)]),
    "hg_batch_info": (
        ctypes.c_int,
        [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64),
         ctypes.POINTER(ctypes.c_double)],
    ),
    "hg_batch_run": (
        ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]
    ),
    "hg_batch_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "hg_prism_adjoint_workspace": (
        ctypes.c_int, [ctypes.c_int64, ctypes.c_int64, ctypes.POINTER(ctypes.c_size_t)]
    ),
    "hg_prism_adjoint": (
        ctypes.c_int,
        [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
         ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_int32, ctypes.c_void_p,
         ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p],
    ),
    "hg_layer_adjoint_workspace": (
        ctypes.c_int,
        [ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, ctypes.POINTER(ctypes.c_size_t)],
    ),
    "hg_layer_adjoint": (
        ctypes.c_int,
        [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
         ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
         ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double, ctypes.c_int32, ctypes.c_void_p,
         ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p],
    ),
    "hg_round_run": (
        ctypes.c_int,
        [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p,
         ctypes.c_void_p],
    ),
    "hg_round_reduce": (
        ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p]
    ),
    "hg_pack_prisms_magnetic": (
        ctypes.c_int,
        [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
         ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p],
    ),
    "hg_prism_magnetic_workspace": (
        ctypes.c_int,
        [ctypes.c_int64, ctypes.c_int64, ctypes.c_int32, ctypes.POINTER(ctypes.c_size_t)],
    ),
    "hg_prism_magnetic": (
        ctypes.c_int,
        [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
         ctypes.c_int64, ctypes.c_int64, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p,
         ctypes.c_size_t, ctypes.c_void_p],
    ),
    "hg_point_forward_workspace": (
        ctypes.c_int, [ctypes.c_int64, ctypes.c_int64, ctypes.POINTER(ctypes.c_size_t)]
    ),
    "hg_point_forward": (
        ctypes.c_int,
        [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
         ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32,
         ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p],
    ),
    "hg_dipole_workspace": (
        ctypes.c_int,
        [ctypes.c_int64, ctypes.c_int64, ctypes.c_int32, ctypes.POINTER(ctypes.c_size_t)],
    ),
    "hg_dipole_magnetic": (
        ctypes.c_int,
        [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
         ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
         ctypes.c_int64, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
         ctypes.c_void_p],
    ),
    "hg_eqs_jacobian": (
        ctypes.c_int,
        [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
         ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32, ctypes.c_void_p,
         ctypes.c_void_p],
    ),
    "hg_eqs_predict": (
        ctypes.c_int,
        [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
         ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32,
         ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p],
    ),
    "hg_tesseroid_forward_workspace": (
        ctypes.c_int, [ctypes.c_int64, ctypes.c_int64, ctypes.POINTER(ctypes.c_size_t)]
    ),
    "hg_tesseroid_forward": (
        ctypes.c_int,
        [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
         ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64, ctypes.c_int32, ctypes.c_int32,
         ctypes.c_int32,
         ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
         ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p],
    ),
    "hg_tesseroid_inside": (
        ctypes.c_int,
        [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
         ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p],
    ),
    "hg_prism_forward_noalloc": (
        ctypes.c_int,
        [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
         ctypes.c_int64, ctypes.c_int64, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p,
         ctypes.c_void_p],
    ),
    "hg_layer_forward_workspace": (
        ctypes.c_int,
        [ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, ctypes.c_uint32,
         ctypes.POINTER(ctypes.c_size_t)],
    ),
    "hg_layer_forward": (
        ctypes.c_int,
        [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
         ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p,
         ctypes.c_void_p, ctypes.c_double, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p,
         ctypes.c_size_t, ctypes.c_void_p],
    ),
}


def lib():
    """Return the loaded native library; raise if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"harmonica_gb300 native library not found at {LIB_PATH}; "
                "build it with harmonica_gb300.build() (needs nvcc)"
            )
        handle = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in PROTOTYPES.items():
            fn = getattr(handle, name)
            fn.restype = res
            fn.argtypes = args
        _lib = handle
    return _lib


class NativeError(RuntimeError):
    """Error reported by the native library through its return code."""


def check(rc):
    if rc != 0:
        msg = lib().hg_last_error()
        raise NativeError(f"harmonica_gb300 native call failed ({rc}): {msg.decode()}")
