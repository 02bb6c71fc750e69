"""
Generate ``reference_point_spherical.npz``: outputs of harmonica's own
``point_gravity`` (src/harmonica/_forward/point.py) in spherical coordinates
-- the potential and g_z kernels there (``potential_spherical``,
``gravity_u_spherical`` over ``distance_spherical_core`` of
_forward/utils.py) are harmonica code, not choclo's -- run from the
reference sources on small seeded cases.

numba and choclo are not installed here.  ``numba.jit`` is replaced by the
identity decorator and ``numba.prange`` by ``range``, which leaves every
arithmetic step unchanged.  From choclo only
``choclo.constants.GRAVITATIONAL_CONST`` (6.6743e-11) is used on this path;
the Cartesian choclo kernels, which it never calls, are placeholders.  The
package ``__init__`` files are not executed; the module is loaded from its
file.

Run from the repository root:
    python tests/golden/make_point_golden.py REFERENCE_ROOT
"""

import importlib
import os
import sys
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
    sys.modules.update({"numba": numba, "choclo": choclo, "choclo.constants": constants,
                        "choclo.point": point})
    src = os.path.join(root, "src", "harmonica")
    for name, path in {"harmonica": src,
                       "harmonica._forward": os.path.join(src, "_forward")}.items():
        pkg = types.ModuleType(name)
        pkg.__path__ = [path]
        sys.modules[name] = pkg
    return importlib.import_module("harmonica._forward.point")


def cases():
    """Observation points and point masses in (longitude, latitude, radius)."""
    rng = np.random.default_rng(20240712)
    n_obs, n_masses = 30, 20
    obs = np.stack([rng.uniform(-30, 30, n_obs), rng.uniform(-60, 60, n_obs),
                    MEAN_RADIUS + rng.uniform(0, 10e3, n_obs)])
    # masses right below some of the points (same longitude and latitude),
    # close to others and spread over the sphere, at depths of 0.1-100 km
    masses_lon = np.concatenate([obs[0, :4], obs[0, 4:8] + 0.01, rng.uniform(-180, 180, 12)])
    masses_lat = np.concatenate([obs[1, :4], obs[1, 4:8] - 0.01, rng.uniform(-89, 89, 12)])
    masses_r = np.concatenate([obs[2, :4] - 100.0, obs[2, 4:8] - 1e3,
                               MEAN_RADIUS - rng.uniform(1e3, 100e3, 12)])
    masses = np.stack([masses_lon, masses_lat, masses_r])
    values = rng.uniform(1e10, 1e13, n_masses)
    return obs, masses, values


def main():
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {sys.argv[0]} REFERENCE_ROOT (the harmonica source tree)")
    root = sys.argv[1]
    point = load_reference(root)
    obs, masses, values = cases()
    out = {"coordinates": obs, "points": masses, "masses": values}
    for field in ("potential", "g_z"):
        out[field] = point.point_gravity(tuple(obs), tuple(masses), values, field,
                                         coordinate_system="spherical", parallel=False)
    path = os.path.join(HERE, "reference_point_spherical.npz")
    np.savez_compressed(path, **out)
    print(f"wrote {path}")


if __name__ == "__main__":
    main()
