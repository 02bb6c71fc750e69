"""
Generate ``mp_truth.npz``: prism fields evaluated with 50 significant digits
(``oracle/mp_check.py``, the closed form of Nagy et al. 2000/2002 that
harmonica's per-pair kernels evaluate, gravity.py:160-164), so that the GPU
tests can measure the error of the CUDA path against the exact values on the
GPU machine, where mpmath is not installed.  Values are in harmonica units
(potential J/kg, accelerations mGal, tensor components Eotvos) for the FP64
inputs stored beside them; NaN marks the singular points of a tensor
component, where the reference returns NaN (gravity.py:141-158; the oracle
decides which points those are).

Three groups, every field:

* ``single_*``: one prism at one point, for three prism shapes and points at
  0.3, 5, 50 and 300 km from the prism centre in generic directions (classes
  in ``single_class``, km).  The closed form cancels more the further the
  point is, so these measure the rounding error of an implementation.
* ``faces_*``: one prism and 125 points on its face planes, on the lines of
  its edges (outside the prism) and at its vertices: the limit conventions.
* ``layer_*``: 64 stations x 64 prisms of the 1e6-prism topography layer (an
  8 x 8 block of prisms at its centre, with its grid, and 48 stations over
  the block plus 16 spread over the survey), the fields summed over the 64
  prisms.  ``layer_easting``/``layer_northing`` and the grids let the test
  rebuild the block as a prism layer; the prism bounds are those the layer
  path computes (centre -/+ half the spacing of the block's first two
  centres, layer.py:582-585).

Run from the repository root:
    python tests/golden/make_mp_golden.py --out tests/golden/mp_truth.npz
(about a minute; needs mpmath).  Nothing is read from the reference: the
inputs are seeded here and the values come from the 50-digit evaluation.
"""

import argparse
import os
import sys
import warnings

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from harmonica_gb300 import synthetic  # noqa: E402
from oracle import mp_check, prism_oracle  # noqa: E402

FIELDS = ("potential", "g_e", "g_n", "g_z", "g_ee", "g_nn", "g_zz", "g_en", "g_ez", "g_nz")
DPS = 50


def single_cases(rng):
    shapes = [(50.0, 70.0, 100.0), (200.0, 200.0, 9000.0), (1000.0, 500.0, 2000.0)]
    prisms, points, which, klass = [], [], [], []
    for k, (dx, dy, dz) in enumerate(shapes):
        w, s = rng.uniform(-500, 500, 2)
        b = -rng.uniform(dz, dz + 3000)
        prisms.append([w, w + dx, s, s + dy, b, b + dz])
        centre = np.array([w + dx / 2, s + dy / 2, b + dz / 2])
        for dist_km in (0.3, 5.0, 50.0, 300.0):
            for _ in range(4):
                # a generic direction: no component near zero (no field
                # component vanishes by symmetry), never below the prism top
                while True:
                    d = rng.normal(size=3)
                    d /= np.linalg.norm(d)
                    if np.all(np.abs(d) > 0.2) and d[2] > 0:
                        break
                p = centre + dist_km * 1e3 * d
                if p[2] <= b + dz:  # at 0.3 km from a tall prism: stay above its top
                    p[2] = b + dz + 50.0
                points.append(p)
                which.append(k)
                klass.append(dist_km)
    return (np.array(prisms), rng.uniform(1800, 3100, len(shapes)), np.array(points),
            np.array(which), np.array(klass))


def face_points():
    prism = np.array([-10.0, 20.0, -5.0, 15.0, -40.0, -10.0])
    pts = [(e, n, u) for e in (-10.0, 20.0, 5.0, -30.0, 40.0)
           for n in (-5.0, 15.0, 3.0, -25.0, 35.0)
           for u in (-40.0, -10.0, -20.0, 5.0, -60.0)]
    return prism, 1000.0, np.array(pts)


def layer_block(rng):
    L = synthetic.layer_topography_1e6()
    j0, k0 = 496, 500  # an 8 x 8 block at the centre of the 1000 x 1000 grid
    easting = L["easting"][j0:j0 + 8].copy()
    northing = L["northing"][k0:k0 + 8].copy()
    top = L["top"][k0:k0 + 8, j0:j0 + 8].copy()
    bottom = L["bottom"][k0:k0 + 8, j0:j0 + 8].copy()
    density = L["density"][k0:k0 + 8, j0:j0 + 8].copy()
    he, hn = (easting[1] - easting[0]) / 2, (northing[1] - northing[0]) / 2
    ge, gn = np.meshgrid(easting, northing)
    prisms = np.column_stack([ge.ravel() - he, ge.ravel() + he, gn.ravel() - hn,
                              gn.ravel() + hn, bottom.ravel(), top.ravel()])
    # 48 stations of the survey nearest the block's centre, 16 spread over it
    se, sn, su = L["coordinates"]
    ce, cn = easting.mean(), northing.mean()
    near = np.argsort((se - ce) ** 2 + (sn - cn) ** 2)[:48]
    far = rng.choice(se.size, 16, replace=False)
    idx = np.concatenate([near, far])
    points = np.column_stack([se[idx], sn[idx], su[idx]])
    return dict(easting=easting, northing=northing, top=top, bottom=bottom, density=density,
                prisms=prisms, points=points)


def truth(field, points, prisms, density):
    """Sums over prisms at each point, 50 digits; NaN where the oracle is NaN."""
    coords = (points[:, 0], points[:, 1], points[:, 2])
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        ora = prism_oracle.prism_gravity(coords, prisms, density, field, disable_checks=True)
    out = np.empty(points.shape[0])
    for i, pt in enumerate(points):
        if np.isnan(ora[i]):
            out[i] = np.nan
            continue
        out[i] = mp_check.prism_gravity(field, [pt], prisms, density, dps=DPS)[0]
    return out


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--out", required=True, help="path of the .npz to write")
    args = ap.parse_args()
    prism_oracle.build_oracle()
    rng = np.random.default_rng(2024)
    data = {"dps": np.array(DPS)}
    sp, sd, spts, which, klass = single_cases(rng)
    data.update(single_prisms=sp, single_density=sd, single_points=spts, single_which=which,
                single_class=klass)
    fp, frho, fpts = face_points()
    data.update(faces_prism=fp, faces_density=np.array(frho), faces_points=fpts)
    blk = layer_block(rng)
    data.update({f"layer_{k}": v for k, v in blk.items()})
    for field in FIELDS:
        data[f"single_{field}"] = np.array([
            mp_check.prism_gravity(field, [spts[i]], [sp[which[i]]], [sd[which[i]]], dps=DPS)[0]
            for i in range(spts.shape[0])])
        data[f"faces_{field}"] = truth(field, fpts, fp[None, :], np.array([frho]))
        data[f"layer_{field}"] = truth(field, blk["points"], blk["prisms"],
                                       blk["density"].ravel())
        print(field, "done", flush=True)
    np.savez_compressed(args.out, **data)


if __name__ == "__main__":
    main()
