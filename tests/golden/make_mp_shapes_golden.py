"""
Generate ``mp_truth_shapes.npz``: the ten prism fields of needles, plates and
slabs (one extent 0.5-1 m, the others up to 2 km) evaluated with 50
significant digits (``oracle/mp_check.py``, the closed form of Nagy et al.
2000/2002 that harmonica's per-pair kernels evaluate, gravity.py:160-164).
Thin prisms are where the regrouped edge and face terms weight their
logarithms and angles by bounds and extents of very different sizes, and
where the per-vertex FP64 sum cancels most for a given distance.

One prism per shape; points at 0.1, 1 and 10 km from the prism centre in
generic directions (four per distance, classes in ``shape_class``, km),
plus four points 2 m from the middle of one of the prism's large faces
(class 0).  Values are in harmonica units (potential J/kg, accelerations
mGal, tensor components Eotvos) for the FP64 inputs stored beside them.

Run from the repository root:
    python tests/golden/make_mp_shapes_golden.py --out tests/golden/mp_truth_shapes.npz
(a few seconds; needs mpmath).  Nothing is read from the reference: the
inputs are seeded here and the values come from the 50-digit evaluation.
"""

import argparse
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import mp_check  # noqa: E402

FIELDS = ("potential", "g_e", "g_n", "g_z", "g_ee", "g_nn", "g_zz", "g_en", "g_ez", "g_nz")
DPS = 50
SHAPES = [(0.5, 500.0, 50.0), (500.0, 0.5, 50.0), (500.0, 50.0, 0.5), (2000.0, 2000.0, 1.0),
          (1.0, 1.0, 2000.0), (0.5, 2000.0, 0.5)]


def generic_direction(rng):
    """A unit vector with no component near zero (no field component vanishes
    by symmetry), pointing upward."""
    while True:
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        if np.all(np.abs(d) > 0.2) and d[2] > 0:
            return d


def cases(rng):
    prisms, points, which, klass = [], [], [], []
    for k, (dx, dy, dz) in enumerate(SHAPES):
        w, s = rng.uniform(-300, 300, 2)
        b = rng.uniform(-600, -10)
        prisms.append([w, w + dx, s, s + dy, b, b + dz])
        centre = np.array([w + dx / 2, s + dy / 2, b + dz / 2])
        thin = int(np.argmin((dx, dy, dz)))  # the axis normal to the large faces
        for _ in range(4):
            # 2 m off a large face, over its middle half
            p = centre.copy()
            for a, ext in enumerate((dx, dy, dz)):
                if a != thin:
                    p[a] += rng.uniform(-0.25, 0.25) * ext
            p[thin] += (dx, dy, dz)[thin] / 2 + 2.0
            points.append(p)
            which.append(k)
            klass.append(0.0)
        for dist_km in (0.1, 1.0, 10.0):
            for _ in range(4):
                points.append(centre + dist_km * 1e3 * generic_direction(rng))
                which.append(k)
                klass.append(dist_km)
    return (np.array(prisms), rng.uniform(1800, 3100, len(SHAPES)), np.array(points),
            np.array(which), np.array(klass))


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--out", required=True, help="path of the .npz to write")
    args = ap.parse_args()
    rng = np.random.default_rng(77)
    prisms, density, points, which, klass = cases(rng)
    data = {"dps": np.array(DPS), "shape_prisms": prisms, "shape_density": density,
            "shape_points": points, "shape_which": which, "shape_class": klass}
    for field in FIELDS:
        data[f"shape_{field}"] = np.array([
            mp_check.prism_gravity(field, [points[i]], [prisms[which[i]]],
                                   [density[which[i]]], dps=DPS)[0]
            for i in range(points.shape[0])])
        print(field, "done", flush=True)
    np.savez_compressed(args.out, **data)


if __name__ == "__main__":
    main()
