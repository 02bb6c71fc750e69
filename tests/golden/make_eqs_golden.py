"""
Generate ``reference_eqs.npz``: outputs of harmonica's own equivalent-source
Jacobian and prediction loops (src/harmonica/_equivalent_sources/utils.py
``jacobian`` and ``predict``) with its Green's functions
(``greens_func_cartesian`` in cartesian.py, ``greens_func_spherical`` in
spherical.py, over ``distance_cartesian`` / ``distance_spherical`` of
_forward/utils.py), run from the reference sources on small seeded cases.

numba, bordado and verde are not installed here.  ``numba.jit`` is replaced
by the identity decorator and ``numba.prange`` by ``range``, which leaves
every arithmetic step unchanged; bordado and verde are only used by the
estimators' gridding and fitting methods, which this script does not call,
so empty modules stand in for them (with an empty class for verde's
``BaseGridder``, which the estimator classes derive from).  The package
``__init__`` files are not executed (they import packages that are absent);
the modules are loaded from their files.

Run from the repository root:
    python tests/golden/make_eqs_golden.py REFERENCE_ROOT
"""

import importlib
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def load_reference(root):
    numba = types.ModuleType("numba")

    def jit(*args, **kwargs):
        if len(args) == 1 and callable(args[0]) and not kwargs:
            return args[0]
        return lambda f: f

    numba.jit = jit
    numba.njit = jit
    numba.prange = range
    verde = types.ModuleType("verde")
    verde_base = types.ModuleType("verde.base")
    verde_base.BaseGridder = type("BaseGridder", (), {})  # base class of the estimators
    verde.base = verde_base
    sys.modules.update({"numba": numba, "bordado": types.ModuleType("bordado"),
                        "verde": verde, "verde.base": verde_base})
    src = os.path.join(root, "src", "harmonica")
    packages = {"harmonica": src, "harmonica._forward": os.path.join(src, "_forward"),
                "harmonica._equivalent_sources": os.path.join(src, "_equivalent_sources")}
    for name, path in packages.items():
        pkg = types.ModuleType(name)
        pkg.__path__ = [path]
        sys.modules[name] = pkg
    utils = importlib.import_module("harmonica._equivalent_sources.utils")
    cartesian = importlib.import_module("harmonica._equivalent_sources.cartesian")
    spherical = importlib.import_module("harmonica._equivalent_sources.spherical")
    return utils, cartesian.greens_func_cartesian, spherical.greens_func_spherical


def cases():
    """Cartesian and spherical data points, sources and coefficients."""
    rng = np.random.default_rng(20240705)
    n_data, n_src = 40, 25
    cart_data = np.stack([rng.uniform(-5e3, 5e3, n_data), rng.uniform(-4e3, 6e3, n_data),
                          rng.uniform(0.0, 300.0, n_data)])
    # sources under a few of the data points (close pairs) and scattered deeper ones
    cart_src = np.stack([np.concatenate([cart_data[0, :5], rng.uniform(-6e3, 6e3, n_src - 5)]),
                         np.concatenate([cart_data[1, :5], rng.uniform(-5e3, 7e3, n_src - 5)]),
                         np.concatenate([cart_data[2, :5] - 50.0,
                                         rng.uniform(-3e3, -500.0, n_src - 5)])])
    radius = 6371008.8
    sph_data = np.stack([rng.uniform(-70, -40, n_data), rng.uniform(-40, -10, n_data),
                         radius + rng.uniform(0, 5e3, n_data)])
    sph_src = np.stack([np.concatenate([sph_data[0, :5], rng.uniform(-72, -38, n_src - 5)]),
                        np.concatenate([sph_data[1, :5], rng.uniform(-42, -8, n_src - 5)]),
                        np.concatenate([sph_data[2, :5] - 500.0,
                                        radius - rng.uniform(1e3, 50e3, n_src - 5)])])
    coefs = rng.normal(0.0, 1e6, n_src)
    return cart_data, cart_src, sph_data, sph_src, coefs


def main():
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {sys.argv[0]} REFERENCE_ROOT (the harmonica source tree)")
    root = sys.argv[1]
    utils, green_cart, green_sph = load_reference(root)
    cart_data, cart_src, sph_data, sph_src, coefs = cases()
    out = {"cart_data": cart_data, "cart_src": cart_src, "sph_data": sph_data,
           "sph_src": sph_src, "coefs": coefs}
    for name, data, src, green in (("cart", cart_data, cart_src, green_cart),
                                   ("sph", sph_data, sph_src, green_sph)):
        jac = np.zeros((data.shape[1], src.shape[1]))
        utils.jacobian(tuple(data), tuple(src), jac, green)
        pred = np.zeros(data.shape[1])
        utils.predict(tuple(data), tuple(src), coefs, pred, green)
        out[f"{name}_jacobian"] = jac
        out[f"{name}_predict"] = pred
    path = os.path.join(HERE, "reference_eqs.npz")
    np.savez_compressed(path, **out)
    print(f"wrote {path}")


if __name__ == "__main__":
    main()
