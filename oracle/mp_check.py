"""
High-precision (mpmath) evaluation of the prism kernels — TEST INFRASTRUCTURE ONLY.

Evaluates the same closed form as ``prism_oracle.c`` (Nagy et al. 2000/2002;
the 8-vertex sum of harmonica's choclo kernels, called from
``src/harmonica/_forward/prisms/gravity.py:524-537``) with 50 significant
digits, so that the rounding error of any FP64 implementation can be measured
against it.  Used to arbitrate when two FP64 implementations disagree near
the 1e-8 level (distant prisms, where the alternating vertex sum cancels).

Raw kernels: SI units, upward z, before harmonica's sign flip and unit
scaling.  Only points off the singular edges/vertices are supported.
"""

import mpmath as mp

G = mp.mpf("6.6743e-11")


def _log_plus_r(a, b, c, r):
    if a >= 0:
        return mp.log(a + r)
    bc2 = b * b + c * c
    if bc2 == 0:
        return -mp.log(r - a)
    return mp.log(bc2 / (r - a))


def _coef_log(coef, a, b, c, r):
    if coef == 0:
        return mp.mpf(0)
    return coef * _log_plus_r(a, b, c, r)


def _coef_atan(coef, a, b, c, r):
    if coef == 0 or a == 0:
        return mp.mpf(0)
    return coef * mp.atan(b * c / (a * r))


def _face_atan(a, b, c, r, upper):
    bc = b * c
    if a != 0:
        return mp.atan(bc / (a * r))
    if bc == 0:
        return mp.mpf(0)
    s = 1 if bc > 0 else -1
    return -s * mp.pi / 2 if upper else s * mp.pi / 2


def _vertex(field, x, y, z, i, j, k):
    r = mp.sqrt(x * x + y * y + z * z)
    if field == "potential":
        return (
            _coef_log(x * y, z, x, y, r)
            + _coef_log(y * z, x, y, z, r)
            + _coef_log(z * x, y, z, x, r)
            - _coef_atan(x * x / 2, x, y, z, r)
            - _coef_atan(y * y / 2, y, z, x, r)
            - _coef_atan(z * z / 2, z, x, y, r)
        )
    if field == "g_e":
        return _coef_log(y, z, x, y, r) + _coef_log(z, y, z, x, r) - _coef_atan(x, x, y, z, r)
    if field == "g_n":
        return _coef_log(z, x, y, z, r) + _coef_log(x, z, x, y, r) - _coef_atan(y, y, z, x, r)
    if field == "g_z":
        return _coef_log(x, y, z, x, r) + _coef_log(y, x, y, z, r) - _coef_atan(z, z, x, y, r)
    if field == "g_ee":
        return -_face_atan(x, y, z, r, i)
    if field == "g_nn":
        return -_face_atan(y, z, x, r, j)
    if field == "g_zz":
        return -_face_atan(z, x, y, r, k)
    if field == "g_en":
        return _log_plus_r(z, x, y, r)
    if field == "g_ez":
        return _log_plus_r(y, z, x, r)
    if field == "g_nz":
        return _log_plus_r(x, y, z, r)
    raise ValueError(field)


def prism_kernel(field, point, prism, density, dps=50):
    """Raw kernel of one prism at one point with `dps` significant digits."""
    with mp.workdps(dps):
        e, n, u = (mp.mpf(float(v)) for v in point)
        p = [mp.mpf(float(v)) for v in prism]
        xs = (p[0] - e, p[1] - e)
        ys = (p[2] - n, p[3] - n)
        zs = (p[4] - u, p[5] - u)
        total = mp.mpf(0)
        for i in range(2):
            for j in range(2):
                for k in range(2):
                    sign = 1 if (i + j + k) % 2 == 1 else -1
                    total += sign * _vertex(field, xs[i], ys[j], zs[k], i, j, k)
        pref = G * mp.mpf(float(density))
        if field in ("g_e", "g_n", "g_z"):
            pref = -pref
        return pref * total


SCALE = {
    "potential": 1.0,
    "g_e": 1e5,
    "g_n": 1e5,
    "g_z": -1e5,
    "g_ee": 1e9,
    "g_nn": 1e9,
    "g_zz": 1e9,
    "g_en": 1e9,
    "g_ez": -1e9,
    "g_nz": -1e9,
}


def prism_gravity(field, points, prisms, densities, dps=50):
    """Harmonica-unit sums over prisms for each point (slow; small cases only)."""
    out = []
    with mp.workdps(dps):
        for pt in points:
            acc = mp.mpf(0)
            for pr, rho in zip(prisms, densities):
                acc += prism_kernel(field, pt, pr, rho, dps)
            out.append(float(acc * SCALE[field]))
    return out
