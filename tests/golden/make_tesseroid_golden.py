"""
Generate ``reference_tesseroid.npz`` and ``reference_tesseroid_variable.npz``:
outputs of harmonica's own tesseroid forward model
(src/harmonica/_forward/tesseroid_gravity.py, _tesseroid_utils.py and
_tesseroid_variable_density.py, run from the reference sources) on small
cases, constant densities and density functions.

numba and choclo are not installed here, so the reference functions are run
as plain Python: ``numba.jit`` is replaced by the identity decorator and
``numba.prange`` by ``range``, which leaves every arithmetic step of the
reference unchanged (numba compiles the same operations).  From choclo only
``choclo.constants.GRAVITATIONAL_CONST`` (6.6743e-11) is used by the
tesseroid path; the choclo point kernels, which it never calls, are
placeholders.  ``harmonica/__init__.py`` is not executed (it imports
packages that are absent); the ``harmonica._forward`` modules are loaded
from their files.

Run from the repository root:
    python tests/golden/make_tesseroid_golden.py REFERENCE_ROOT
"""

import os
import sys
import time
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# Earth's mean radius (IUGG, metres); any radius of this size serves.
MEAN_RADIUS = 6371008.8


def load_reference(root):
    numba = types.ModuleType("numba")

    def jit(*args, **kwargs):
        if len(args) == 1 and callable(args[0]) and not kwargs:
            return args[0]
        return lambda f: f

    numba.jit = jit
    numba.njit = jit
    numba.prange = range
    sys.modules["numba"] = numba

    choclo = types.ModuleType("choclo")
    constants = types.ModuleType("choclo.constants")
    constants.GRAVITATIONAL_CONST = 6.6743e-11
    point = types.ModuleType("choclo.point")

    def _unused(*args, **kwargs):
        raise NotImplementedError

    for name in ("gravity_e", "gravity_ee", "gravity_en", "gravity_eu", "gravity_n",
                 "gravity_nn", "gravity_nu", "gravity_pot", "gravity_u", "gravity_uu"):
        setattr(point, name, _unused)
    choclo.constants, choclo.point = constants, point
    sys.modules.update({"choclo": choclo, "choclo.constants": constants, "choclo.point": point})

    src = os.path.join(root, "src", "harmonica")
    pkg = types.ModuleType("harmonica")
    pkg.__path__ = [src]
    fwd = types.ModuleType("harmonica._forward")
    fwd.__path__ = [os.path.join(src, "_forward")]
    sys.modules.update({"harmonica": pkg, "harmonica._forward": fwd})
    import importlib  # noqa: PLC0415

    tg = importlib.import_module("harmonica._forward.tesseroid_gravity")
    tu = importlib.import_module("harmonica._forward._tesseroid_utils")
    return tg, tu


def shell_tesseroids(shape, bottom, top):
    longitude = np.linspace(0, 360, shape[0] + 1)
    latitude = np.linspace(-90, 90, shape[1] + 1)
    return np.array([
        [w, e, s, n, bottom, top]
        for w, e in zip(longitude[:-1], longitude[1:])
        for s, n in zip(latitude[:-1], latitude[1:])
    ])


def cases():
    """(name, coordinates (3, n), tesseroids (m, 6), density (m,), radial, disable_checks)."""
    out = []
    r = MEAN_RADIUS
    # the single-tesseroid gallery example (doc/gallery_src/forward/tesseroid.py), coarser grid
    lon, lat = np.meshgrid(np.linspace(-80, -40, 7), np.linspace(-50, -10, 6))
    out.append(("gallery", np.stack([lon.ravel(), lat.ravel(), np.full(lon.size, r + 100e3)]),
                np.array([[-70, -50, -40, -20, r - 10e3, r]], dtype=float), np.array([2670.0]),
                False, False))
    # w > e tesseroid made continuous (test/test_tesseroid.py:444-462)
    out.append(("continuity", np.array([[0.0], [0.0], [r + 1e3]]),
                np.array([[350, 10, -10, 10, r - 1e4, r]], dtype=float), np.array([1e3]),
                False, False))
    # seeded irregular model: 10 tesseroids, 12 points 0.5-60 km above them
    rng = np.random.default_rng(20240611)
    tess = []
    for _ in range(10):
        w = rng.uniform(-20, 15)
        s = rng.uniform(-20, 15)
        top = r - rng.uniform(0, 2e3)
        tess.append([w, w + rng.uniform(0.5, 5), s, s + rng.uniform(0.5, 5),
                     top - rng.uniform(1e3, 40e3), top])
    tess = np.array(tess)
    dens = rng.uniform(-500, 3000, size=10)
    pts = np.stack([rng.uniform(-22, 22, 12), rng.uniform(-22, 22, 12),
                    r + rng.uniform(500, 60e3, 12)])
    out.append(("random", pts, tess, dens, False, False))
    out.append(("random_radial", pts, tess, dens, True, False))
    # spherical shell, 3D discretisation (test/test_tesseroid.py:729-770), one thickness
    out.append(("shell3d", np.array([[0.0], [0.0], [r + 1e3]]),
                shell_tesseroids((6, 6), r - 1e3, r), np.full(36, 1000.0), True, False))
    # spherical shell, 2D discretisation with points on its top surface
    # (test/test_tesseroid.py:683-726), three points, one thickness
    out.append(("shell2d_surface", np.array([[0.0, 125.0, 250.0], [0.0, 40.0, -80.0],
                                             [r, r, r]]),
                shell_tesseroids((12, 6), r - 100.0, r), np.full(72, 1000.0), False, False))
    # bottom > top with checks disabled (test/test_tesseroid.py:224-244)
    out.append(("disable_checks", np.array([[0.0], [0.0], [10.0]]),
                np.array([[0.0, 10.0, 0.0, 10.0, 20.0, 10.0]]), np.array([100.0]), False, True))
    return out


# density functions of the variable-density cases (test/test_tesseroid_variable_density.py
# fixtures); tests/test_gpu_tesseroid.py defines the same functions
def quadratic_density(radius):
    return 1e-3 * (radius - 3e3) ** 2 + 1900.0


def linear_shell_density(top, bottom):
    slope = (2500.0 - 3300.0) / (top - bottom)
    constant = 2500.0 - slope * top
    return lambda radius: slope * radius + constant


def exponential_shell_density(top, bottom, b_factor):
    thickness = top - bottom
    a_factor = (3300.0 - 2670.0) / (1 - np.exp(-b_factor))
    constant = 3300.0 - a_factor
    return lambda radius: a_factor * np.exp(-b_factor * (radius - bottom) / thickness) + constant


def variable_shell(bottom, top, shape=(6, 12)):
    n_lat, n_lon = shape
    longitude = np.linspace(-180, 180, n_lon + 1)
    latitude = np.linspace(-90, 90, n_lat + 1)
    return np.array([[w, e, s, n, bottom, top]
                     for w, e in zip(longitude[:-1], longitude[1:])
                     for s, n in zip(latitude[:-1], latitude[1:])])


def variable_cases():
    """(name, coordinates, tesseroids, density function)."""
    top = 6371e3
    bottom = top - 1e3
    shell = variable_shell(bottom, top)
    pts = np.array([[10.0, -35.0, 120.0, 10.0, -35.0, 120.0],
                    [5.0, 42.0, -61.0, 5.0, 42.0, -61.0],
                    [top + 1e3, top + 5e3, top + 20e3, top, top, top]])
    single = np.array([[-3.0, 3.0, -2.0, 2.0, 5400e3, 6300e3]])
    spts = np.array([[0.0, 2.5, -4.0], [0.0, 1.0, 3.5], [6300e3, 6300e3 + 1e3, 6300e3 + 50e3]])
    return [
        ("linear_shell", pts, shell, linear_shell_density(top, bottom)),
        ("exponential_shell", pts, shell, exponential_shell_density(top, bottom, 5)),
        ("single_constant_fn", spts, single, lambda radius: 2900.0),
    ]


def main(root):
    tg, tu = load_reference(root)
    import importlib  # noqa: PLC0415

    tv = importlib.import_module("harmonica._forward._tesseroid_variable_density")
    var = {}
    var_names = []
    for name, coords, tess, fn in variable_cases():
        for field in ("potential", "g_z"):
            t0 = time.time()
            res = tg.tesseroid_gravity(tuple(coords), tess, fn, field=field, parallel=False)
            key = f"{name}_{field}"
            var_names.append(key)
            var[f"{key}_coords"] = coords
            var[f"{key}_tesseroids"] = tess
            var[f"{key}_result"] = np.asarray(res, dtype=np.float64).ravel()
            print(f"{key}: {time.time() - t0:.2f} s", file=sys.stderr)
    # density-based discretization of single tesseroids
    var["split_quadratic"] = np.array(
        tv._density_based_discretization((-3, 2, -4, 5, 2e3, 5e3), quadratic_density), dtype=float)
    for b in (5, 100):
        t = (0.0, 30.0, 0.0, 30.0, 6371e3 - 1e3, 6371e3)
        var[f"split_exponential_{b}"] = np.array(
            tv._density_based_discretization(t, exponential_shell_density(t[5], t[4], b)),
            dtype=float)
    var["names"] = np.array(var_names)
    np.savez_compressed(os.path.join(HERE, "reference_tesseroid_variable.npz"), **var)
    store = {}
    names = []
    for name, coords, tess, dens, radial, disable in cases():
        for field in ("potential", "g_z"):
            t0 = time.time()
            res = tg.tesseroid_gravity(
                tuple(coords), tess, dens, field=field, parallel=False,
                radial_adaptive_discretization=radial, disable_checks=disable,
            )
            key = f"{name}_{field}"
            names.append(key)
            store[f"{key}_coords"] = coords
            store[f"{key}_tesseroids"] = tess
            store[f"{key}_density"] = dens
            store[f"{key}_flags"] = np.array([int(radial), int(disable)])
            store[f"{key}_result"] = np.asarray(res, dtype=np.float64).ravel()
            print(f"{key}: {time.time() - t0:.2f} s", file=sys.stderr)
    # small tesseroids of one pair, in the reference's order
    # (test/test_tesseroid.py:642-660); with the radial split the same pair
    # overflows the stack, which is recorded as an empty array
    stack = np.empty((tg.STACK_SIZE, 6))
    small = np.empty((tg.MAX_DISCRETIZATIONS, 6))
    tess = np.array([-10.0, 10.0, -10.0, 10.0, 1.0, 10.0])
    for radial in (False, True):
        try:
            n = tu._adaptive_discretization(np.array([0.0, 0.0, 10.0]), tess, 10, stack, small,
                                            radial)
            store[f"split_radial{int(radial)}"] = small[:n].copy()
        except OverflowError as err:
            print(f"radial={radial}: {err}", file=sys.stderr)
            store[f"split_radial{int(radial)}"] = np.empty((0, 6))
    store["names"] = np.array(names)
    path = os.path.join(HERE, "reference_tesseroid.npz")
    np.savez_compressed(path, **store)
    print(f"wrote {path}", file=sys.stderr)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {sys.argv[0]} REFERENCE_ROOT (the harmonica source tree)")
    main(sys.argv[1])
