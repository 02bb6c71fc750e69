"""
Generate the golden fixtures in this directory.

1. ``reference_doctests.json``: the numbers harmonica itself prints in its
   doctests, read from the reference sources:
     * src/harmonica/_forward/prisms/gravity.py:170-193 (g_z of one and two
       prisms at three points, printed to 5 decimals);
     * src/harmonica/_forward/prisms/layer.py:111-118 (layer boundaries and
       get_prism).
   The inputs are those of the doctests; the expected outputs are parsed from
   the ``print`` results in the reference file, so the fixture is the
   reference's own output.
2. ``reference_point_potential.npz``: the reference's point-mass potential
   samples (test/data/sample_point_gravity.csv).
3. ``oracle_small.npz``: outputs of the CPU oracle (oracle/prism_oracle.c) for
   the TestAgainstChoclo fixture of the reference tests
   (test/test_prism.py:161-190) for all ten fields, and for a small seeded
   prism layer, kept as regression vectors for the oracle and the GPU path.

Run from the repository root:  python tests/golden/make_golden.py REFERENCE_ROOT
"""

import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import prism_oracle  # noqa: E402


def parse_doctests(ref_root):
    grav = open(os.path.join(ref_root, "src/harmonica/_forward/prisms/gravity.py")).read()
    tuples = re.findall(r"^\s*\((-?\d+\.\d+), (-?\d+\.\d+), (-?\d+\.\d+)\)\s*$", grav, re.M)
    assert len(tuples) == 2, tuples
    layer = open(os.path.join(ref_root, "src/harmonica/_forward/prisms/layer.py")).read()
    lists = re.findall(r"^\s*\[(-?[\d.]+(?:, -?[\d.]+)+)\]\s*$", layer, re.M)
    assert len(lists) == 2, lists
    return {
        "source": "harmonica doctests: src/harmonica/_forward/prisms/gravity.py:170-193, "
        "src/harmonica/_forward/prisms/layer.py:95-118",
        "decimals": 5,
        "coordinates": [[-40, 0, 40], [0, 0, 0], [30, 30, 30]],
        "single_prism": {
            "prisms": [[-34, 5, -18, 14, -345, -146]],
            "density": [2670],
            "g_z": [float(v) for v in tuples[0]],
        },
        "two_prisms": {
            "prisms": [[-134, -5, -45, 45, -200, -50], [5, 134, -45, 45, -180, -30]],
            "density": [-300, 300],
            "g_z": [float(v) for v in tuples[1]],
        },
        "layer": {
            "easting": [0, 2.5, 5, 7.5, 10],
            "northing": [2, 4, 6, 8],
            "surface": "arange(20).reshape(4, 5)",
            "reference": 0,
            "boundaries": [float(v) for v in lists[0].split(",")],
            "get_prism_0_2": [float(v) for v in lists[1].split(",")],
        },
    }


def choclo_fixture():
    # test/test_prism.py:167-190
    prisms = np.array(
        [[-10, 10, -10, 0, -10, 0], [-10, 0, -10, 10, -20, -10], [5, 15, 5, 15, -15, -5]],
        dtype=float,
    )
    densities = np.array([400, -200, 300], dtype=float)
    coords = (
        np.array([-5, 10, 0, 15], dtype=float),
        np.array([14, -4, 11, 0], dtype=float),
        np.array([9, 6, 6, 12], dtype=float),
    )
    return coords, prisms, densities


def small_layer():
    rng = np.random.default_rng(11)
    easting = np.linspace(0, 9000, 10)
    northing = np.linspace(0, 7000, 8)
    top = rng.uniform(-500, 800, (8, 10))
    bottom = np.full((8, 10), -3000.0)
    density = rng.uniform(2000, 3000, (8, 10))
    ge, gn = np.meshgrid(np.linspace(-1000, 10000, 7), np.linspace(-1000, 8000, 6))
    gu = np.full_like(ge, 1000.0)
    return easting, northing, bottom, top, density, (ge.ravel(), gn.ravel(), gu.ravel())


def point_sample(ref_root):
    """The reference's own point-mass potential samples (test/data/sample_point_gravity.csv:
    a 5000 kg mass at the origin, used by test/test_point_gravity.py:131-154)."""
    data = np.loadtxt(os.path.join(ref_root, "test", "data", "sample_point_gravity.csv"),
                      delimiter=",")
    np.savez(os.path.join(HERE, "reference_point_potential.npz"), easting=data[:, 0],
             northing=data[:, 1], upward=data[:, 2], potential=data[:, 3],
             point=np.zeros(3), mass=np.array([5000.0]))


def main():
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {sys.argv[0]} REFERENCE_ROOT (the harmonica source tree)")
    ref_root = sys.argv[1]
    if os.path.isdir(ref_root):
        with open(os.path.join(HERE, "reference_doctests.json"), "w") as f:
            json.dump(parse_doctests(ref_root), f, indent=1)
        point_sample(ref_root)
    coords, prisms, densities = choclo_fixture()
    arrays = {
        "choclo_e": coords[0],
        "choclo_n": coords[1],
        "choclo_u": coords[2],
        "choclo_prisms": prisms,
        "choclo_density": densities,
    }
    for field in prism_oracle.FIELDS:
        arrays[f"choclo_{field}"] = prism_oracle.prism_gravity(coords, prisms, densities, field)
    easting, northing, bottom, top, density, lc = small_layer()
    arrays.update(
        layer_easting=easting,
        layer_northing=northing,
        layer_bottom=bottom,
        layer_top=top,
        layer_density=density,
        layer_obs_e=lc[0],
        layer_obs_n=lc[1],
        layer_obs_u=lc[2],
    )
    for field in prism_oracle.FIELDS:
        arrays[f"layer_{field}"] = prism_oracle.layer_gravity(
            lc, easting, northing, bottom, top, density, field
        )
    np.savez(os.path.join(HERE, "oracle_small.npz"), **arrays)


if __name__ == "__main__":
    main()
