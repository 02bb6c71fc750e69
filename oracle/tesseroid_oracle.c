/*
 * CPU oracle for the tesseroid gravity forward model -- TEST INFRASTRUCTURE
 * ONLY.  Only tests/, __graft_entry__.smoke() and the CPU-baseline leg of
 * bench.py call it; the product library never links it.
 *
 * Plain C restatement of harmonica's adaptive Gauss-Legendre quadrature for
 * tesseroids of constant density, in the same arithmetic order as the
 * reference so that the two agree to the last bits on the same libm:
 *
 *   - jit_tesseroid_gravity            src/harmonica/_forward/tesseroid_gravity.py:236-333
 *     (per point: loop over tesseroids, adaptive discretisation, GLQ of
 *     every small tesseroid in discovery order; sign and mGal at :209-215)
 *   - _adaptive_discretization         src/harmonica/_forward/_tesseroid_utils.py:150-241
 *     (stack of STACK_SIZE=100 tesseroids, split test distance / size <
 *     ratio, OverflowError on a full stack or more than
 *     MAX_DISCRETIZATIONS=100000 small tesseroids)
 *   - _split_tesseroid                 _tesseroid_utils.py:244-263
 *   - _tesseroid_dimensions            _tesseroid_utils.py:266-280
 *   - _distance_tesseroid_point        _tesseroid_utils.py:283-295, with
 *     distance_spherical / distance_spherical_core  src/harmonica/_forward/utils.py:122-201
 *   - gauss_legendre_quadrature        _tesseroid_utils.py:18-115
 *   - potential_spherical, gravity_u_spherical   src/harmonica/_forward/point.py:323-354
 *
 * Degrees are converted with x * (pi / 180), as numpy.radians does.
 * Compiled with -ffp-contract=off (no fused multiply-adds), like numba's
 * default code generation.
 */
#include <math.h>
#include <stdint.h>
#include <string.h>

#define TESS_STACK_SIZE 100
#define TESS_MAX_DISCRETIZATIONS 100000
#define TESS_OK 0
#define TESS_STACK_OVERFLOW 1
#define TESS_TOO_MANY 2

/* choclo.constants.GRAVITATIONAL_CONST, the value harmonica's point kernels use. */
static const double G_CONST = 6.6743e-11;

static const double PI_ = 3.141592653589793238462643383279502884;

/*
 * Conditioning probe (tests only).  When set nonzero, every cos, sin and acos
 * result of this file is moved by -1, 0 or +1 ulp, chosen by a hash of its
 * argument: the size of the change in the result measures how much the
 * reference's own output depends on the last bit of its libm.  Zero (the
 * default) leaves the functions untouched.
 */
static int trig_perturbation = 0;

void oracle_set_trig_perturbation(int on) { trig_perturbation = on; }

static double nudge(double v, double arg, uint64_t salt)
{
    if (!trig_perturbation) return v;
    uint64_t u;
    memcpy(&u, &arg, sizeof u);
    u = (u ^ salt) * 0x9E3779B97F4A7C15ull;
    const int step = (int)((u >> 61) % 3) - 1;
    return step == 0 ? v : nextafter(v, step > 0 ? INFINITY : -INFINITY);
}

static double t_cos(double x) { return nudge(cos(x), x, 1); }
static double t_sin(double x) { return nudge(sin(x), x, 2); }
static double t_acos(double x) { return nudge(acos(x), x, 3); }

static double radians(double deg) { return deg * (PI_ / 180.0); }

/* distance_spherical_core (utils.py:164-201): distance and cos(psi). */
static double distance_core(double longitude, double cosphi, double sinphi, double radius,
                            double longitude_p, double cosphi_p, double sinphi_p,
                            double radius_p, double *cospsi_out)
{
    const double coslambda = t_cos(longitude_p - longitude);
    const double cospsi = sinphi_p * sinphi + cosphi_p * cosphi * coslambda;
    const double dr = radius - radius_p;
    if (cospsi_out) *cospsi_out = cospsi;
    return sqrt(dr * dr + 2 * radius * radius_p * (1 - cospsi));
}

/* potential_spherical / gravity_u_spherical (point.py:323-354). */
static double point_kernel(int field, double longitude, double cosphi, double sinphi,
                           double radius, double longitude_p, double cosphi_p,
                           double sinphi_p, double radius_p)
{
    double cospsi;
    const double dist = distance_core(longitude, cosphi, sinphi, radius, longitude_p, cosphi_p,
                                      sinphi_p, radius_p, &cospsi);
    if (field == 0) return 1 / dist * G_CONST;
    const double delta_z = radius - radius_p * cospsi;
    /* distance**3 as numpy evaluates it for a float64 scalar (pow) */
    return -G_CONST * delta_z / pow(dist, 3);
}

/* _tesseroid_dimensions (_tesseroid_utils.py:266-280). */
void oracle_tesseroid_dimensions(const double *t, double *out3)
{
    const double w = radians(t[0]), e = radians(t[1]);
    const double s = radians(t[2]), n = radians(t[3]);
    const double top = t[5];
    const double latc = (n + s) / 2;
    const double l_lat = top * t_acos(t_sin(n) * t_sin(s) + t_cos(n) * t_cos(s));
    const double sl = t_sin(latc), cl = t_cos(latc);
    const double l_lon = top * t_acos(sl * sl + cl * cl * t_cos(e - w));
    out3[0] = l_lon;
    out3[1] = l_lat;
    out3[2] = top - t[4];
}

/* distance_spherical (utils.py:122-160) between a point and the tesseroid
 * centre (_tesseroid_utils.py:283-295); coordinates in degrees/metres. */
double oracle_distance_tesseroid_point(double longitude, double latitude, double radius,
                                       const double *t)
{
    const double lon_p = radians((t[0] + t[1]) / 2);
    const double lat_p = radians((t[2] + t[3]) / 2);
    const double r_p = (t[4] + t[5]) / 2;
    const double lat = radians(latitude);
    return distance_core(radians(longitude), t_cos(lat), t_sin(lat), radius, lon_p, t_cos(lat_p),
                         t_sin(lat_p), r_p, 0);
}

/* gauss_legendre_quadrature (_tesseroid_utils.py:18-115).  nodes/weights:
 * [lon(2), lat(2), rad(2)] from numpy.polynomial.legendre.leggauss(2). */
double oracle_tesseroid_glq(int field, double longitude_rad, double cosphi, double sinphi,
                            double radius, const double *t, const double *density,
                            const double *nodes, const double *weights)
{
    /* density[k]: the density at radial node k -- one value twice for
     * gauss_legendre_quadrature, the density function at radius_p for
     * gauss_legendre_quadrature_variable_density
     * (_tesseroid_variable_density.py:18-107) */
    const double w = t[0], e = t[1], s = t[2], n = t[3], bottom = t[4], top = t[5];
    const double a_factor = 1.0 / 8 * radians(e - w) * radians(n - s) * (top - bottom);
    double result = 0.0;
    for (int j = 0; j < 2; j++) {
        const double latitude_p = radians(0.5 * (n - s) * nodes[2 + j] + 0.5 * (n + s));
        const double cosphi_p = t_cos(latitude_p);
        const double sinphi_p = t_sin(latitude_p);
        for (int k = 0; k < 2; k++) {
            const double radius_p = 0.5 * (top - bottom) * nodes[4 + k] + 0.5 * (top + bottom);
            const double kappa = radius_p * radius_p * cosphi_p;
            for (int i = 0; i < 2; i++) {
                const double longitude_p = radians(0.5 * (e - w) * nodes[i] + 0.5 * (e + w));
                const double mass =
                    density[k] * a_factor * kappa * weights[i] * weights[2 + j] * weights[4 + k];
                result += mass * point_kernel(field, longitude_rad, cosphi, sinphi, radius,
                                              longitude_p, cosphi_p, sinphi_p, radius_p);
            }
        }
    }
    return result;
}

/* _split_tesseroid (_tesseroid_utils.py:244-263): push the children in
 * (lon, lat, rad) loop order. */
static int split(const double *t, int n_lon, int n_lat, int n_rad, double (*stack)[6], int top)
{
    const double d_lon = (t[1] - t[0]) / n_lon;
    const double d_lat = (t[3] - t[2]) / n_lat;
    const double d_rad = (t[5] - t[4]) / n_rad;
    for (int i = 0; i < n_lon; i++)
        for (int j = 0; j < n_lat; j++)
            for (int k = 0; k < n_rad; k++) {
                top++;
                stack[top][0] = t[0] + d_lon * i;
                stack[top][1] = t[0] + d_lon * (i + 1);
                stack[top][2] = t[2] + d_lat * j;
                stack[top][3] = t[2] + d_lat * (j + 1);
                stack[top][4] = t[4] + d_rad * k;
                stack[top][5] = t[4] + d_rad * (k + 1);
            }
    return top;
}

/*
 * _adaptive_discretization (_tesseroid_utils.py:150-241) for one point and
 * one tesseroid.  Each small tesseroid is handed to ``leaf`` in the order
 * the reference stores it in ``small_tesseroids`` (which is also the order
 * it integrates them).  ``stack_size`` / ``max_leaves`` default to the
 * reference's STACK_SIZE / MAX_DISCRETIZATIONS when <= 0.  Returns the
 * number of small tesseroids, or -TESS_STACK_OVERFLOW / -TESS_TOO_MANY.
 */
typedef void (*leaf_fn)(const double *t, void *ctx);

static int64_t adaptive(const double *point, const double *tess, double ratio, int radial,
                        int stack_size, int64_t max_leaves, leaf_fn leaf, void *ctx)
{
    double stack[TESS_STACK_SIZE][6];
    if (stack_size <= 0 || stack_size > TESS_STACK_SIZE) stack_size = TESS_STACK_SIZE;
    if (max_leaves <= 0) max_leaves = TESS_MAX_DISCRETIZATIONS;
    for (int c = 0; c < 6; c++) stack[0][c] = tess[c];
    int top = 0;
    int64_t n_splits = 0;
    while (top >= 0) {
        double t[6];
        for (int c = 0; c < 6; c++) t[c] = stack[top][c];
        top--;
        double l[3];
        oracle_tesseroid_dimensions(t, l);
        const double distance = oracle_distance_tesseroid_point(point[0], point[1], point[2], t);
        int n_lon = 1, n_lat = 1, n_rad = 1;
        if (distance / l[0] < ratio) n_lon = 2;
        if (distance / l[1] < ratio) n_lat = 2;
        if (distance / l[2] < ratio && radial) n_rad = 2;
        if (n_lon * n_lat * n_rad > 1) {
            if ((top + 1) + n_lon * n_lat * n_rad > stack_size) return -TESS_STACK_OVERFLOW;
            top = split(t, n_lon, n_lat, n_rad, stack, top);
        } else {
            if (n_splits + 1 > max_leaves) return -TESS_TOO_MANY;
            if (leaf) leaf(t, ctx);
            n_splits++;
        }
    }
    return n_splits;
}

typedef struct {
    double *out;     /* small tesseroids, 6 per row (or NULL) */
    int64_t cap;
    int64_t n;
} collect_ctx;

static void collect_leaf(const double *t, void *vctx)
{
    collect_ctx *c = (collect_ctx *)vctx;
    if (c->out && c->n < c->cap)
        for (int k = 0; k < 6; k++) c->out[6 * c->n + k] = t[k];
    c->n++;
}

/* The small tesseroids of one (point, tesseroid) pair, for the unit tests. */
int64_t oracle_adaptive_discretization(const double *point, const double *tess, double ratio,
                                       int radial, int stack_size, int64_t max_leaves,
                                       double *out, int64_t cap)
{
    collect_ctx c = {out, cap, 0};
    return adaptive(point, tess, ratio, radial, stack_size, max_leaves, collect_leaf, &c);
}

typedef struct {
    int field;
    double longitude_rad, cosphi, sinphi, radius;
    double density[2];
    const double *nodes, *weights;
    double acc;
} glq_ctx;

static void glq_leaf(const double *t, void *vctx)
{
    glq_ctx *g = (glq_ctx *)vctx;
    g->acc += oracle_tesseroid_glq(g->field, g->longitude_rad, g->cosphi, g->sinphi, g->radius, t,
                                   g->density, g->nodes, g->weights);
}

/*
 * jit_tesseroid_gravity (tesseroid_gravity.py:236-333) without the final
 * sign/unit step: result[i] = sum over tesseroids and their small
 * tesseroids of the GLQ point masses (field 0 potential, 1 radial
 * acceleration g_u in SI).  ``tesseroids``: n_tess rows of
 * (w, e, s, n, bottom, top), already checked and with null tesseroids
 * removed.  Returns TESS_OK or the first overflow code met.
 */
int oracle_tesseroid_gravity(int field, int radial, int64_t n_obs, const double *longitude,
                             const double *latitude, const double *radius, int64_t n_tess,
                             const double *tesseroids, const double *density,
                             int density_per_node, const double *nodes, const double *weights,
                             double *result, int parallel)
{
    /* density: one value per tesseroid, or (density_per_node, 2D
     * discretization only) the density at its two radial nodes */
    const double ratio = field == 0 ? 1.0 : 2.5;
    int status = TESS_OK;
#pragma omp parallel for schedule(dynamic, 1) if (parallel)
    for (int64_t i = 0; i < n_obs; i++) {
        const double point[3] = {longitude[i], latitude[i], radius[i]};
        const double lat = radians(latitude[i]);
        glq_ctx g = {field, radians(longitude[i]), t_cos(lat), t_sin(lat), radius[i], {0.0, 0.0},
                     nodes, weights, 0.0};
        double acc = 0.0;
        for (int64_t j = 0; j < n_tess; j++) {
            g.density[0] = density_per_node ? density[2 * j] : density[j];
            g.density[1] = density_per_node ? density[2 * j + 1] : density[j];
            /* result[i] += glq(leaf) leaf by leaf, as the reference does */
            g.acc = acc;
            const int64_t rc = adaptive(point, tesseroids + 6 * j, ratio, radial, 0, 0, glq_leaf, &g);
            if (rc < 0) {
#pragma omp atomic write
                status = (int)(-rc);
                break;
            }
            acc = g.acc;
        }
        result[i] = acc;
    }
    return status;
}
