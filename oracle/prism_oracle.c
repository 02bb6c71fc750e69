/*
 * CPU oracle for the right-rectangular-prism gravity forward model.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker that the CUDA path in
 * harmonica_gb300/csrc is compared against; nothing in the product links or
 * calls it.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg load the library built from it.
 *
 * What it restates (harmonica, paths relative to the harmonica project):
 *   - the all-pairs loop of jit_prism_gravity
 *       src/harmonica/_forward/prisms/gravity.py:489-540
 *     (parallel over observation points, sequential over prisms, in prism
 *     order, out[i] += kernel(...));
 *   - the prism-layer loop of _forward_gravity_prism_layer
 *       src/harmonica/_forward/prisms/layer.py:522-625
 *     (easting columns outer, northing rows inner, boundaries generated from
 *     the centres +- half spacing, skipping prisms with zero/NaN density,
 *     thickness below the threshold, or NaN top/bottom);
 *   - the singular-point predicates used by _check_singular_points
 *       src/harmonica/_forward/prisms/gravity.py:239-449.
 *
 * The per-pair kernels live in the third-party package choclo
 * (choclo.prism.gravity_pot/e/n/u/ee/nn/uu/en/eu/nu, imported at
 * gravity.py:14-25; dependency "choclo >= 0.1", pyproject.toml:41, not
 * vendored).  Its source is not available, so the kernels below are written
 * from the published closed form of Nagy, Papp & Benedek (2000, J. Geodesy 74,
 * 552; corrections 2002) with observation-relative vertex coordinates, as the
 * reference docstring cites (gravity.py:160-164), and with the conventions the
 * reference documents at gravity.py:141-158:
 *   - potential and acceleration are finite everywhere;
 *   - tensor components are NaN on the singular edges/vertices of each
 *     component;
 *   - diagonal tensor components on a face normal to their direction take the
 *     limit approached from outside the prism.
 *
 * Units and signs are those of the raw kernels: SI, upward z.  The caller
 * (oracle/prism_oracle.py) applies harmonica's sign flip and unit scaling
 * (gravity.py:227-236).
 *
 * Field codes: 0 potential, 1 g_e, 2 g_n, 3 g_z(upward kernel), 4 g_ee,
 * 5 g_nn, 6 g_zz, 7 g_en, 8 g_ez, 9 g_nz.
 */
#include <math.h>
#include <stdint.h>

#define ORACLE_G 6.6743e-11 /* harmonica constants.py:12 */

/*
 * ln(a + r) with r = sqrt(a^2 + b^2 + c^2).
 * For a < 0 the sum a + r cancels; use (a + r)(r - a) = b^2 + c^2 instead.
 * When b = c = 0 and a < 0 the exact value is ln(0); the ln(b^2 + c^2) part
 * is then dropped.  It is identical for the two vertices of the same edge line
 * (same b, c, opposite vertex signs), so it cancels in the 8-vertex sum unless
 * the observation point lies on the edge itself, which is a singular point
 * reported as NaN by the tensor kernels and multiplied by a zero coefficient in
 * the potential and acceleration kernels.
 */
static double log_plus_r(double a, double b, double c, double r)
{
    if (a >= 0.0) return log(a + r);
    double bc2 = b * b + c * c;
    if (bc2 == 0.0) return -log(r - a);
    return log(bc2 / (r - a));
}

/* coef * ln(a + r) with the limit coef -> 0 taken as 0. */
static double coef_log(double coef, double a, double b, double c, double r)
{
    if (coef == 0.0) return 0.0;
    return coef * log_plus_r(a, b, c, r);
}

/* coef * atan(b c / (a r)); the limit for coef = a -> 0 is 0. */
static double coef_atan(double coef, double a, double b, double c, double r)
{
    if (coef == 0.0 || a == 0.0) return 0.0;
    return coef * atan(b * c / (a * r));
}

/*
 * atan(b c / (a r)) for the diagonal tensor kernels.  At a == 0 (observation
 * point on the plane of a face normal to this axis) the value is the limit
 * from outside the prism: for the lower bound of the axis (upper == 0) the
 * outside side is a -> 0+, for the upper bound (upper == 1) it is a -> 0-.
 */
static double face_atan(double a, double b, double c, double r, int upper)
{
    double bc = b * c;
    if (a != 0.0) return atan(bc / (a * r));
    if (bc == 0.0) return 0.0;
    double half_pi = 1.5707963267948966;
    double s = bc > 0.0 ? 1.0 : -1.0;
    return upper ? -s * half_pi : s * half_pi;
}

/* One vertex term of each field (before the density and G prefactor). */
static double vertex_term(int field, double x, double y, double z, int i, int j, int k)
{
    double r = sqrt(x * x + y * y + z * z);
    switch (field) {
    case 0: /* potential: K(x,y,z) */
        return coef_log(x * y, z, x, y, r) + coef_log(y * z, x, y, z, r) +
               coef_log(z * x, y, z, x, r) - coef_atan(0.5 * x * x, x, y, z, r) -
               coef_atan(0.5 * y * y, y, z, x, r) - coef_atan(0.5 * z * z, z, x, y, r);
    case 1: /* dK/dx */
        return coef_log(y, z, x, y, r) + coef_log(z, y, z, x, r) - coef_atan(x, x, y, z, r);
    case 2: /* dK/dy */
        return coef_log(z, x, y, z, r) + coef_log(x, z, x, y, r) - coef_atan(y, y, z, x, r);
    case 3: /* dK/dz */
        return coef_log(x, y, z, x, r) + coef_log(y, x, y, z, r) - coef_atan(z, z, x, y, r);
    case 4: /* d2K/dx2 */
        return -face_atan(x, y, z, r, i);
    case 5: /* d2K/dy2 */
        return -face_atan(y, z, x, r, j);
    case 6: /* d2K/dz2 */
        return -face_atan(z, x, y, r, k);
    case 7: /* d2K/dxdy */
        return log_plus_r(z, x, y, r);
    case 8: /* d2K/dxdz */
        return log_plus_r(y, z, x, r);
    case 9: /* d2K/dydz */
        return log_plus_r(x, y, z, r);
    default:
        return NAN;
    }
}

/* Singular-edge predicates (closed intervals, so vertices are included). */
static int on_easting_edge(double e, double n, double u, const double *p)
{
    return (n == p[2] || n == p[3]) && (u == p[4] || u == p[5]) && p[0] <= e && e <= p[1];
}
static int on_northing_edge(double e, double n, double u, const double *p)
{
    return (e == p[0] || e == p[1]) && (u == p[4] || u == p[5]) && p[2] <= n && n <= p[3];
}
static int on_upward_edge(double e, double n, double u, const double *p)
{
    return (e == p[0] || e == p[1]) && (n == p[2] || n == p[3]) && p[4] <= u && u <= p[5];
}

/* 1 if the observation point is a singular point of `field` for prism p. */
int oracle_is_singular(int field, double e, double n, double u, const double *p)
{
    switch (field) {
    case 4: return on_northing_edge(e, n, u, p) || on_upward_edge(e, n, u, p);
    case 5: return on_easting_edge(e, n, u, p) || on_upward_edge(e, n, u, p);
    case 6: return on_easting_edge(e, n, u, p) || on_northing_edge(e, n, u, p);
    case 7: return on_upward_edge(e, n, u, p);
    case 8: return on_northing_edge(e, n, u, p);
    case 9: return on_easting_edge(e, n, u, p);
    default: return 0;
    }
}

/*
 * Raw kernel of one prism p = [w, e, s, n, b, t] with density rho at one
 * observation point: G rho times the signed 8-vertex sum, SI units, upward z.
 */
double oracle_prism_kernel(int field, double e, double n, double u, const double *p, double rho)
{
    if (field >= 4 && oracle_is_singular(field, e, n, u, p)) return NAN;
    double xs[2] = {p[0] - e, p[1] - e};
    double ys[2] = {p[2] - n, p[3] - n};
    double zs[2] = {p[4] - u, p[5] - u};
    double sum = 0.0;
    for (int i = 0; i < 2; i++)
        for (int j = 0; j < 2; j++)
            for (int k = 0; k < 2; k++) {
                double sign = ((i + j + k) % 2 == 1) ? 1.0 : -1.0;
                /* (1,1,1) -> +, (0,0,0) -> -: upper bound minus lower bound */
                sum += sign * vertex_term(field, xs[i], ys[j], zs[k], i, j, k);
            }
    /* d/d(observation) = -d/d(vertex) for the three first derivatives */
    double pref = ORACLE_G * rho;
    if (field >= 1 && field <= 3) pref = -pref;
    return pref * sum;
}

/*
 * out[i] += sum_j kernel(station i, prism j), prisms as an (m, 6) row-major
 * array [w, e, s, n, b, t].  Mirrors gravity.py:524-537.
 */
void oracle_prism_gravity(int field, int64_t n_obs, const double *easting, const double *northing,
                          const double *upward, int64_t n_prisms, const double *prisms,
                          const double *density, double *out, int n_threads)
{
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 16) num_threads(n_threads > 0 ? n_threads : 1)
#endif
    for (int64_t i = 0; i < n_obs; i++) {
        double acc = out[i];
        for (int64_t j = 0; j < n_prisms; j++)
            acc += oracle_prism_kernel(field, easting[i], northing[i], upward[i], prisms + 6 * j,
                                       density[j]);
        out[i] = acc;
    }
    (void)n_threads;
}

/*
 * Prism-layer forward, mirroring layer.py:582-625: easting index j outer,
 * northing index k inner, boundaries from the centres +- half spacing, and the
 * skips for zero/NaN density, thickness below `threshold`, NaN top/bottom.
 * bottom, top and density are (n_north, n_east) row-major.
 */
void oracle_layer_gravity(int field, int64_t n_obs, const double *easting, const double *northing,
                          const double *upward, int64_t n_east, int64_t n_north,
                          const double *centre_e, const double *centre_n, const double *bottom,
                          const double *top, const double *density, double threshold, double *out,
                          int n_threads)
{
    double half_e = (centre_e[1] - centre_e[0]) / 2.0;
    double half_n = (centre_n[1] - centre_n[0]) / 2.0;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 16) num_threads(n_threads > 0 ? n_threads : 1)
#endif
    for (int64_t i = 0; i < n_obs; i++) {
        double acc = out[i];
        for (int64_t j = 0; j < n_east; j++) {
            double w = centre_e[j] - half_e, e = centre_e[j] + half_e;
            for (int64_t k = 0; k < n_north; k++) {
                double rho = density[k * n_east + j];
                if (rho == 0.0 || isnan(rho)) continue;
                double b = bottom[k * n_east + j], t = top[k * n_east + j];
                if (t - b < threshold) continue;
                if (isnan(t) || isnan(b)) continue;
                double p[6] = {w, e, centre_n[k] - half_n, centre_n[k] + half_n, b, t};
                acc += oracle_prism_kernel(field, easting[i], northing[i], upward[i], p, rho);
            }
        }
        out[i] = acc;
    }
    (void)n_threads;
}

/*
 * All ten raw kernels of one prism at one point at once, each equal bit for
 * bit to oracle_prism_kernel(field, ...): the three logs ln(a + r) and the
 * three arctangents of a vertex are the same expressions for every field
 * (vertex_term), so they are evaluated once per vertex and combined per
 * field in the same operation order; the vertex sums run in the same order.
 */
static void prism_kernel_all(double e, double n, double u, const double *p, double rho,
                             double out[10])
{
    double xs[2] = {p[0] - e, p[1] - e};
    double ys[2] = {p[2] - n, p[3] - n};
    double zs[2] = {p[4] - u, p[5] - u};
    double sum[10] = {0.0};
    for (int i = 0; i < 2; i++)
        for (int j = 0; j < 2; j++)
            for (int k = 0; k < 2; k++) {
                double sign = ((i + j + k) % 2 == 1) ? 1.0 : -1.0;
                double x = xs[i], y = ys[j], z = zs[k];
                double r = sqrt(x * x + y * y + z * z);
                double lz = log_plus_r(z, x, y, r); /* ln(z + r) */
                double lx = log_plus_r(x, y, z, r); /* ln(x + r) */
                double ly = log_plus_r(y, z, x, r); /* ln(y + r) */
                double ax = x == 0.0 ? 0.0 : atan(y * z / (x * r));
                double ay = y == 0.0 ? 0.0 : atan(z * x / (y * r));
                double az = z == 0.0 ? 0.0 : atan(x * y / (z * r));
#define CL(coef, l) ((coef) == 0.0 ? 0.0 : (coef) * (l))
#define CA(coef, a) ((coef) == 0.0 ? 0.0 : (coef) * (a))
                double t[10];
                t[0] = CL(x * y, lz) + CL(y * z, lx) + CL(z * x, ly) - CA(0.5 * x * x, ax) -
                       CA(0.5 * y * y, ay) - CA(0.5 * z * z, az);
                t[1] = CL(y, lz) + CL(z, ly) - CA(x, ax);
                t[2] = CL(z, lx) + CL(x, lz) - CA(y, ay);
                t[3] = CL(x, ly) + CL(y, lx) - CA(z, az);
#undef CL
#undef CA
                t[4] = -face_atan(x, y, z, r, i);
                t[5] = -face_atan(y, z, x, r, j);
                t[6] = -face_atan(z, x, y, r, k);
                t[7] = lz;
                t[8] = ly;
                t[9] = lx;
                for (int f = 0; f < 10; f++) sum[f] += sign * t[f];
            }
    for (int f = 0; f < 10; f++) {
        double pref = ORACLE_G * rho;
        if (f >= 1 && f <= 3) pref = -pref;
        out[f] = (f >= 4 && oracle_is_singular(f, e, n, u, p)) ? NAN : pref * sum[f];
    }
}

/*
 * All ten fields of the prism-layer forward (oracle_layer_gravity for every
 * field in one pass, same loop order and skips); out is (10, n_obs).
 */
void oracle_layer_gravity_all(int64_t n_obs, const double *easting, const double *northing,
                              const double *upward, int64_t n_east, int64_t n_north,
                              const double *centre_e, const double *centre_n,
                              const double *bottom, const double *top, const double *density,
                              double threshold, double *out, int n_threads)
{
    double half_e = (centre_e[1] - centre_e[0]) / 2.0;
    double half_n = (centre_n[1] - centre_n[0]) / 2.0;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 4) num_threads(n_threads > 0 ? n_threads : 1)
#endif
    for (int64_t i = 0; i < n_obs; i++) {
        double acc[10];
        for (int f = 0; f < 10; f++) acc[f] = out[f * n_obs + i];
        for (int64_t j = 0; j < n_east; j++) {
            double w = centre_e[j] - half_e, e = centre_e[j] + half_e;
            for (int64_t k = 0; k < n_north; k++) {
                double rho = density[k * n_east + j];
                if (rho == 0.0 || isnan(rho)) continue;
                double b = bottom[k * n_east + j], t = top[k * n_east + j];
                if (t - b < threshold) continue;
                if (isnan(t) || isnan(b)) continue;
                double p[6] = {w, e, centre_n[k] - half_n, centre_n[k] + half_n, b, t};
                double v[10];
                prism_kernel_all(easting[i], northing[i], upward[i], p, rho, v);
                for (int f = 0; f < 10; f++) acc[f] += v[f];
            }
        }
        for (int f = 0; f < 10; f++) out[f * n_obs + i] = acc[f];
    }
    (void)n_threads;
}

/* Serial any-pair singular check with early exit, as gravity.py:272-449. */
int oracle_any_singular(int field, int64_t n_obs, const double *easting, const double *northing,
                        const double *upward, int64_t n_prisms, const double *prisms)
{
    if (field < 4) return 0;
    for (int64_t i = 0; i < n_obs; i++)
        for (int64_t j = 0; j < n_prisms; j++)
            if (oracle_is_singular(field, easting[i], northing[i], upward[i], prisms + 6 * j))
                return 1;
    return 0;
}

/* ------------------------------------------------------------------------
 * Point masses (harmonica src/harmonica/_forward/point.py:357-450): the
 * all-pairs loops of point_mass_cartesian and point_mass_spherical with the
 * kernels written from the formulas of the point_gravity docstring
 * (point.py:125-224): V = G m / l, g = grad V, tensor = grad grad V
 * (choclo.point kernels, SI, upward z; sign/units applied by the caller).
 * Field codes as for prisms.  Spherical: coordinates are longitude (deg),
 * latitude (deg), radius (m); fields 0 (potential) and 3 (g_z) only, the
 * distance is point.py's distance_spherical_core (utils.py:164-201).
 */
static double point_kernel_cart(int field, double e, double n, double u, double ep, double np,
                                double up)
{
    double dx = e - ep, dy = n - np, dz = u - up;
    double l = sqrt(dx * dx + dy * dy + dz * dz);
    double l3 = l * l * l, l5 = l3 * l * l;
    switch (field) {
    case 0: return ORACLE_G / l;
    case 1: return -ORACLE_G * dx / l3;
    case 2: return -ORACLE_G * dy / l3;
    case 3: return -ORACLE_G * dz / l3;
    case 4: return ORACLE_G * (3.0 * dx * dx - l * l) / l5;
    case 5: return ORACLE_G * (3.0 * dy * dy - l * l) / l5;
    case 6: return ORACLE_G * (3.0 * dz * dz - l * l) / l5;
    case 7: return ORACLE_G * 3.0 * dx * dy / l5;
    case 8: return ORACLE_G * 3.0 * dx * dz / l5;
    case 9: return ORACLE_G * 3.0 * dy * dz / l5;
    default: return NAN;
    }
}

void oracle_point_gravity(int field, int spherical, int64_t n_obs, const double *c1,
                          const double *c2, const double *c3, int64_t n_points, const double *p1,
                          const double *p2, const double *p3, const double *masses, double *out,
                          int n_threads)
{
    const double deg = 3.141592653589793 / 180.0;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 16) num_threads(n_threads > 0 ? n_threads : 1)
#endif
    for (int64_t i = 0; i < n_obs; i++) {
        double acc = out[i];
        if (!spherical) {
            for (int64_t j = 0; j < n_points; j++)
                acc += masses[j] * point_kernel_cart(field, c1[i], c2[i], c3[i], p1[j], p2[j],
                                                     p3[j]);
        } else {
            double lon = c1[i] * deg, lat = c2[i] * deg, r = c3[i];
            double cphi = cos(lat), sphi = sin(lat);
            for (int64_t j = 0; j < n_points; j++) {
                double lonp = p1[j] * deg, latp = p2[j] * deg, rp = p3[j];
                double cphip = cos(latp), sphip = sin(latp);
                double coslambda = cos(lonp - lon);
                double cospsi = sphip * sphi + cphip * cphi * coslambda;
                double dist = sqrt((r - rp) * (r - rp) + 2.0 * r * rp * (1.0 - cospsi));
                double k = field == 0 ? ORACLE_G / dist
                                      : -ORACLE_G * (r - rp * cospsi) / (dist * dist * dist);
                acc += masses[j] * k;
            }
        }
        out[i] = acc;
    }
    (void)n_threads;
}

/* ------------------------------------------------------------------------
 * Magnetic prisms (harmonica src/harmonica/_forward/prisms/magnetic.py:275-400,
 * loops over points (parallel) and prisms (sequential)).  choclo's
 * magnetic_field kernel is restated from magnetostatics: outside the prism
 * b = mu0/(4 pi) T M with T_ab the unit-density gradient-tensor 8-vertex sums
 * of this file (vertex_term fields 4..9).  SI (tesla); the caller scales to nT.
 */
static double tensor_kernel(int field, double e, double n, double u, const double *p)
{
    double xs[2] = {p[0] - e, p[1] - e}, ys[2] = {p[2] - n, p[3] - n}, zs[2] = {p[4] - u, p[5] - u};
    double sum = 0.0;
    for (int i = 0; i < 2; i++)
        for (int j = 0; j < 2; j++)
            for (int k = 0; k < 2; k++) {
                double sign = ((i + j + k) % 2 == 1) ? 1.0 : -1.0;
                sum += sign * vertex_term(field, xs[i], ys[j], zs[k], i, j, k);
            }
    return sum;
}

void oracle_prism_magnetic(int64_t n_obs, const double *easting, const double *northing,
                           const double *upward, int64_t n_prisms, const double *prisms,
                           const double *me, const double *mn, const double *mu, double *be,
                           double *bn, double *bu, int n_threads)
{
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 16) num_threads(n_threads > 0 ? n_threads : 1)
#endif
    for (int64_t i = 0; i < n_obs; i++) {
        double se = 0.0, sn = 0.0, su = 0.0;
        for (int64_t j = 0; j < n_prisms; j++) {
            const double *p = prisms + 6 * j;
            double tee = tensor_kernel(4, easting[i], northing[i], upward[i], p);
            double tnn = tensor_kernel(5, easting[i], northing[i], upward[i], p);
            double tuu = tensor_kernel(6, easting[i], northing[i], upward[i], p);
            double ten = tensor_kernel(7, easting[i], northing[i], upward[i], p);
            double teu = tensor_kernel(8, easting[i], northing[i], upward[i], p);
            double tnu = tensor_kernel(9, easting[i], northing[i], upward[i], p);
            se += 1e-7 * (tee * me[j] + ten * mn[j] + teu * mu[j]);
            sn += 1e-7 * (ten * me[j] + tnn * mn[j] + tnu * mu[j]);
            su += 1e-7 * (teu * me[j] + tnu * mn[j] + tuu * mu[j]);
        }
        be[i] += se;
        bn[i] += sn;
        bu[i] += su;
    }
    (void)n_threads;
}
