"""
CPU oracle for the prism gravity forward model — TEST INFRASTRUCTURE ONLY.

This module is the checker for the CUDA path.  Only ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` may
import it; the product package ``harmonica_gb300`` never does.

It restates, in numpy around the C kernels of ``prism_oracle.c``:

* ``prism_gravity``: harmonica ``src/harmonica/_forward/prisms/gravity.py:51-236``
  (field check :196-198, broadcasting :200-205, density/prism checks :207-215,
  ``_discard_null_prisms`` :452-486, accumulation :524-537, sign and units
  :227-236);
* ``check_prisms``: ``src/harmonica/_forward/prisms/utils.py:12-43``;
* ``layer_gravity``: ``DatasetAccessorPrismLayer.gravity``,
  ``src/harmonica/_forward/prisms/layer.py:314-433`` and the loop at :582-625.

The C library is built by ``oracle/Makefile`` (``build_oracle()`` below runs
it).  Results are in harmonica units: potential J/kg, accelerations mGal,
tensor components Eotvos.
"""

import ctypes
import os
import subprocess
import warnings

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libprism_oracle.so")

FIELD_CODES = {
    "potential": 0,
    "g_e": 1,
    "g_n": 2,
    "g_z": 3,
    "g_ee": 4,
    "g_nn": 5,
    "g_zz": 6,
    "g_en": 7,
    "g_ez": 8,
    "g_nz": 9,
}
FIELDS = tuple(FIELD_CODES)

_lib = None


def build_oracle():
    """Compile the C oracle with the Makefile next to this file, one process
    at a time (a file lock in the build folder; make skips an up-to-date
    library, and the library is renamed into place whole)."""
    import fcntl  # noqa: PLC0415

    os.makedirs(os.path.dirname(LIB_PATH), exist_ok=True)
    with open(os.path.join(os.path.dirname(LIB_PATH), ".build.lock"), "w") as handle:
        fcntl.flock(handle, fcntl.LOCK_EX)
        try:
            subprocess.run(["make", "-s", "-C", HERE], check=True)
        finally:
            fcntl.flock(handle, fcntl.LOCK_UN)


def _load():
    global _lib
    if _lib is not None:
        return _lib
    sources = [os.path.join(HERE, f) for f in ("prism_oracle.c", "tesseroid_oracle.c")]
    if not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < max(
        os.path.getmtime(f) for f in sources
    ):
        build_oracle()
    lib = ctypes.CDLL(LIB_PATH)
    dp = ctypes.POINTER(ctypes.c_double)
    i64 = ctypes.c_int64
    lib.oracle_prism_kernel.restype = ctypes.c_double
    lib.oracle_prism_kernel.argtypes = [
        ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double, dp, ctypes.c_double
    ]
    lib.oracle_prism_gravity.restype = None
    lib.oracle_prism_gravity.argtypes = [
        ctypes.c_int, i64, dp, dp, dp, i64, dp, dp, dp, ctypes.c_int
    ]
    lib.oracle_layer_gravity.restype = None
    lib.oracle_layer_gravity.argtypes = [
        ctypes.c_int, i64, dp, dp, dp, i64, i64, dp, dp, dp, dp, dp, ctypes.c_double, dp,
        ctypes.c_int,
    ]
    lib.oracle_layer_gravity_all.restype = None
    lib.oracle_layer_gravity_all.argtypes = [
        i64, dp, dp, dp, i64, i64, dp, dp, dp, dp, dp, ctypes.c_double, dp, ctypes.c_int,
    ]
    lib.oracle_any_singular.restype = ctypes.c_int
    lib.oracle_any_singular.argtypes = [ctypes.c_int, i64, dp, dp, dp, i64, dp]
    lib.oracle_point_gravity.restype = None
    lib.oracle_point_gravity.argtypes = [
        ctypes.c_int, ctypes.c_int, i64, dp, dp, dp, i64, dp, dp, dp, dp, dp, ctypes.c_int
    ]
    lib.oracle_prism_magnetic.restype = None
    lib.oracle_prism_magnetic.argtypes = [
        i64, dp, dp, dp, i64, dp, dp, dp, dp, dp, dp, dp, ctypes.c_int
    ]
    lib.oracle_is_singular.restype = ctypes.c_int
    lib.oracle_is_singular.argtypes = [
        ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double, dp
    ]
    lib.oracle_tesseroid_dimensions.restype = None
    lib.oracle_tesseroid_dimensions.argtypes = [dp, dp]
    lib.oracle_distance_tesseroid_point.restype = ctypes.c_double
    lib.oracle_distance_tesseroid_point.argtypes = [
        ctypes.c_double, ctypes.c_double, ctypes.c_double, dp
    ]
    lib.oracle_tesseroid_glq.restype = ctypes.c_double
    lib.oracle_tesseroid_glq.argtypes = [
        ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double, dp,
        dp, dp, dp,
    ]
    lib.oracle_adaptive_discretization.restype = i64
    lib.oracle_adaptive_discretization.argtypes = [
        dp, dp, ctypes.c_double, ctypes.c_int, ctypes.c_int, i64, dp, i64
    ]
    lib.oracle_set_trig_perturbation.restype = None
    lib.oracle_set_trig_perturbation.argtypes = [ctypes.c_int]
    lib.oracle_tesseroid_gravity.restype = ctypes.c_int
    lib.oracle_tesseroid_gravity.argtypes = [
        ctypes.c_int, ctypes.c_int, i64, dp, dp, dp, i64, dp, dp, ctypes.c_int, dp, dp, dp,
        ctypes.c_int,
    ]
    _lib = lib
    return lib


def _ptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def default_threads():
    return os.cpu_count() or 1


def scale_result(result, field):
    """Sign flip and unit conversion of gravity.py:227-236 (in place)."""
    if field in ("g_z", "g_ez", "g_nz"):
        result *= -1
    if field in ("g_e", "g_n", "g_z"):
        result *= 1e5
    if field in ("g_ee", "g_nn", "g_zz", "g_en", "g_ez", "g_nz"):
        result *= 1e9
    return result


def check_prisms(prisms):
    """Restates utils.py:12-43 (same messages)."""
    west, east, south, north, bottom, top = tuple(prisms[:, i] for i in range(6))
    err_msg = "Invalid prism or prisms. "
    bad_we = west > east
    bad_sn = south > north
    bad_bt = bottom > top
    if bad_we.any():
        err_msg += "The west boundary can't be greater than the east one.\n"
        for prism in prisms[bad_we]:
            err_msg += f"\tInvalid prism: {prism}\n"
        raise ValueError(err_msg)
    if bad_sn.any():
        err_msg += "The south boundary can't be greater than the north one.\n"
        for prism in prisms[bad_sn]:
            err_msg += f"\tInvalid prism: {prism}\n"
        raise ValueError(err_msg)
    if bad_bt.any():
        err_msg += "The bottom boundary can't be greater than the top one.\n"
        for prism in prisms[bad_bt]:
            err_msg += f"\tInvalid tesseroid: {prism}\n"
        raise ValueError(err_msg)


def discard_null_prisms(prisms, density):
    """Restates gravity.py:452-486."""
    west, east, south, north, bottom, top = tuple(prisms[:, i] for i in range(6))
    null = (west == east) | (south == north) | (bottom == top)
    null[density == 0] = True
    keep = np.logical_not(null)
    return prisms[keep, :], density[keep]


def any_singular(coordinates, prisms, field):
    """Serial predicate of gravity.py:239-449 (True if any pair is singular)."""
    lib = _load()
    e, n, u = (_f64(c) for c in coordinates)
    p = _f64(prisms)
    return bool(
        lib.oracle_any_singular(
            FIELD_CODES[field], e.size, _ptr(e), _ptr(n), _ptr(u), p.shape[0], _ptr(p)
        )
    )


def prism_kernel(field, point, prism, density):
    """Raw SI kernel (upward z, no unit scaling) of one prism at one point."""
    lib = _load()
    p = _f64(prism)
    return lib.oracle_prism_kernel(
        FIELD_CODES[field], float(point[0]), float(point[1]), float(point[2]), _ptr(p),
        float(density),
    )


def prism_gravity(
    coordinates,
    prisms,
    density,
    field,
    parallel=True,
    dtype="float64",
    progressbar=False,
    disable_checks=False,
    n_threads=None,
):
    """Oracle restatement of harmonica.prism_gravity (gravity.py:51-236)."""
    if field not in FIELD_CODES:
        raise ValueError(f"Gravitational field {field} not recognized")
    cast = np.broadcast(*coordinates[:3])
    coordinates = tuple(
        _f64(np.broadcast_to(np.asarray(c, dtype=np.float64), cast.shape)).ravel()
        for c in coordinates[:3]
    )
    prisms = np.atleast_2d(np.asarray(prisms, dtype=np.float64))
    density = np.atleast_1d(np.asarray(density, dtype=np.float64)).ravel()
    if not disable_checks:
        if density.size != prisms.shape[0]:
            raise ValueError(
                f"Number of elements in density ({density.size}) "
                + f"mismatch the number of prisms ({prisms.shape[0]})"
            )
        check_prisms(prisms)
        if any_singular(coordinates, prisms, field):
            warnings.warn(
                "Found observation point on singular point of a prism.",
                UserWarning,
                stacklevel=2,
            )
    prisms, density = discard_null_prisms(prisms, density)
    prisms = _f64(prisms)
    density = _f64(density)
    out = np.zeros(cast.size, dtype=np.float64)
    lib = _load()
    e, n, u = coordinates
    threads = (n_threads or default_threads()) if parallel else 1
    lib.oracle_prism_gravity(
        FIELD_CODES[field], e.size, _ptr(e), _ptr(n), _ptr(u), prisms.shape[0], _ptr(prisms),
        _ptr(density), _ptr(out), threads,
    )
    scale_result(out, field)
    return out.astype(dtype).reshape(cast.shape)


def layer_gravity(
    coordinates,
    easting,
    northing,
    bottom,
    top,
    density,
    field,
    thickness_threshold=None,
    parallel=True,
    n_threads=None,
):
    """Oracle restatement of the prism-layer accessor's gravity (layer.py:314-433)."""
    if field not in FIELD_CODES:
        raise ValueError(f"Gravitational field '{field}' not recognized.")
    cast = np.broadcast(*coordinates[:3])
    coordinates = tuple(
        _f64(np.broadcast_to(np.asarray(c, dtype=np.float64), cast.shape)).ravel()
        for c in coordinates[:3]
    )
    easting, northing = _f64(easting), _f64(northing)
    bottom, top, density = _f64(bottom), _f64(top), _f64(density)
    threshold = 0.0 if thickness_threshold is None else float(thickness_threshold)
    out = np.zeros(cast.size, dtype=np.float64)
    lib = _load()
    e, n, u = coordinates
    threads = (n_threads or default_threads()) if parallel else 1
    lib.oracle_layer_gravity(
        FIELD_CODES[field], e.size, _ptr(e), _ptr(n), _ptr(u), easting.size, northing.size,
        _ptr(easting), _ptr(northing), _ptr(bottom), _ptr(top), _ptr(density), threshold,
        _ptr(out), threads,
    )
    scale_result(out, field)
    return out.reshape(cast.shape)


def layer_gravity_fields(coordinates, easting, northing, bottom, top, density,
                         thickness_threshold=None, n_threads=None):
    """All ten fields of ``layer_gravity`` in one pass over the pairs (each
    field equal bit for bit to ``layer_gravity`` of that field); returns a
    dict field -> array in harmonica units."""
    cast = np.broadcast(*coordinates[:3])
    coordinates = tuple(
        _f64(np.broadcast_to(np.asarray(c, dtype=np.float64), cast.shape)).ravel()
        for c in coordinates[:3]
    )
    easting, northing = _f64(easting), _f64(northing)
    bottom, top, density = _f64(bottom), _f64(top), _f64(density)
    threshold = 0.0 if thickness_threshold is None else float(thickness_threshold)
    e, n, u = coordinates
    out = np.zeros((len(FIELDS), e.size), dtype=np.float64)
    _load().oracle_layer_gravity_all(
        e.size, _ptr(e), _ptr(n), _ptr(u), easting.size, northing.size, _ptr(easting),
        _ptr(northing), _ptr(bottom), _ptr(top), _ptr(density), threshold, _ptr(out),
        n_threads or default_threads(),
    )
    result = {}
    for f, code in FIELD_CODES.items():
        row = out[code].copy()
        scale_result(row, f)
        result[f] = row.reshape(cast.shape)
    return result


POINT_FIELDS = {
    "cartesian": {"potential": 0, "g_e": 1, "g_n": 2, "g_z": 3, "g_ee": 4, "g_nn": 5, "g_zz": 6,
                  "g_en": 7, "g_ez": 8, "g_nz": 9, "g_ne": 7, "g_ze": 8, "g_zn": 9},
    "spherical": {"potential": 0, "g_z": 3, "g_n": None, "g_e": None},
}


def point_gravity(coordinates, points, masses, field, coordinate_system="cartesian",
                  parallel=True, dtype="float64", n_threads=None):
    """Oracle restatement of harmonica.point_gravity (point.py:30-268)."""
    if coordinate_system not in ("cartesian", "spherical"):
        raise ValueError(f"Coordinate system {coordinate_system} not recognized.")
    cast = np.broadcast(*coordinates[:3])
    coords = tuple(
        _f64(np.broadcast_to(np.asarray(c, dtype=np.float64), cast.shape)).ravel()
        for c in coordinates[:3]
    )
    pts = tuple(_f64(np.atleast_1d(np.asarray(p, dtype=np.float64)).ravel()) for p in points[:3])
    masses = _f64(np.atleast_1d(np.asarray(masses, dtype=np.float64)).ravel())
    if masses.size != pts[0].size:
        raise ValueError(
            f"Number of elements in masses ({masses.size}) "
            + f"mismatch the number of points ({pts[0].size})"
        )
    table = POINT_FIELDS[coordinate_system]
    if field not in table:
        raise ValueError(f"Gravitational field '{field}' not recognized")
    if table[field] is None:
        raise NotImplementedError
    code = table[field]
    out = np.zeros(cast.size)
    lib = _load()
    threads = (n_threads or default_threads()) if parallel else 1
    lib.oracle_point_gravity(code, int(coordinate_system == "spherical"), out.size,
                             _ptr(coords[0]), _ptr(coords[1]), _ptr(coords[2]), masses.size,
                             _ptr(pts[0]), _ptr(pts[1]), _ptr(pts[2]), _ptr(masses), _ptr(out),
                             threads)
    if field in ("g_z", "g_ez", "g_ze", "g_nz", "g_zn"):
        out *= -1
    if field in ("g_e", "g_n", "g_z"):
        out *= 1e5
    if field in ("g_ee", "g_nn", "g_zz", "g_en", "g_ez", "g_nz", "g_ne", "g_ze", "g_zn"):
        out *= 1e9
    return out.astype(dtype).reshape(cast.shape)


MAGNETIC_FIELDS = ("b", "b_e", "b_n", "b_u")


def prism_magnetic(coordinates, prisms, magnetization, field, parallel=True, dtype=np.float64,
                   disable_checks=False, n_threads=None):
    """Oracle restatement of harmonica.prism_magnetic (magnetic.py:28-136), nT."""
    if field not in MAGNETIC_FIELDS:
        raise ValueError(
            f"Invalid field '{field}'. Please choose one of '{','.join(MAGNETIC_FIELDS)}'."
        )
    cast = np.broadcast(*coordinates[:3])
    coords = tuple(
        _f64(np.broadcast_to(np.asarray(c, dtype=np.float64), cast.shape)).ravel()
        for c in coordinates[:3]
    )
    prisms = np.atleast_2d(np.asarray(prisms, dtype=np.float64))
    mag = tuple(_f64(np.atleast_1d(np.asarray(m, dtype=np.float64)).ravel())
                for m in magnetization)
    if not disable_checks:
        if len(mag) != 3:
            raise ValueError(
                f"Invalid magnetization vectors with '{len(mag)}' elements. "
                + "Magnetization vectors should have only 3 elements."
            )
        if mag[0].size != prisms.shape[0]:
            raise ValueError(
                f"Number of magnetization vectors ({mag[0].size}) "
                + f"mismatch the number of prisms ({prisms.shape[0]})"
            )
        check_prisms(prisms)
    w, e, s, n, b, t = (prisms[:, k] for k in range(6))
    keep = ~((w == e) | (s == n) | (b == t) | ((mag[0] == 0) & (mag[1] == 0) & (mag[2] == 0)))
    prisms = _f64(prisms[keep])
    mag = tuple(_f64(m[keep]) for m in mag)
    out = [np.zeros(cast.size) for _ in range(3)]
    lib = _load()
    threads = (n_threads or default_threads()) if parallel else 1
    lib.oracle_prism_magnetic(cast.size, _ptr(coords[0]), _ptr(coords[1]), _ptr(coords[2]),
                              prisms.shape[0], _ptr(prisms), _ptr(mag[0]), _ptr(mag[1]),
                              _ptr(mag[2]), _ptr(out[0]), _ptr(out[1]), _ptr(out[2]), threads)
    out = [(o * 1e9).astype(dtype).reshape(cast.shape) for o in out]
    if field == "b":
        return tuple(out)
    return out[{"b_e": 0, "b_n": 1, "b_u": 2}[field]]
