// Tesseroid (spherical prism) gravity of constant-density tesseroids:
// harmonica src/harmonica/_forward/tesseroid_gravity.py:35-333 with the
// adaptive discretisation and Gauss-Legendre quadrature of
// src/harmonica/_forward/_tesseroid_utils.py:18-295.
//
// Work decomposition.  One thread per computation point; tesseroids in
// shared-memory tiles; grid = point tiles x tesseroid chunks, chunk partials
// reduced in fixed order (as for the prisms).  A prepare kernel computes,
// once per tesseroid, everything of the reference's per-pair work that does
// not depend on the point: the size of the tesseroid (_tesseroid_dimensions),
// its centre, and the 8 Gauss-Legendre point masses (positions and masses of
// gauss_legendre_quadrature).  A pair whose tesseroid needs no split (the
// common case away from the points) then costs the distance to the centre
// and the 8 point-mass kernels.  A pair that needs splitting is queued in a
// per-warp list in shared memory and later run by one lane with the
// reference's stack algorithm (stack of 100, split order, small tesseroids
// integrated in discovery order), so that the lanes of a warp share the
// expensive pairs instead of idling behind one of them.  Queued pairs are
// added to their point's sum in list order: results are deterministic.
//
// Arithmetic.  The split decisions follow the reference's operation order
// in FP64 without contraction into fused multiply-adds (__dmul_rn /
// __dadd_rn), so they differ from the reference only through the last bits
// of cos/sin/acos; so do the point-mass positions and masses of every
// tesseroid (glq_nodes).  The split test distance / size < ratio is
// evaluated exactly whenever an FP32 pre-test on the Cartesian distance to
// the centre, with a rigorous error margin, does not already prove "no
// split".  The point masses are summed by glq_sum_pairs on float pairs
// packed two nodes per float2 (FFMA2/FADD2/FMUL2): the Cartesian difference
// of the point and each node (48-bit coordinates), 1 / l from a float-pair
// reciprocal square root, and for g_z the radial component
// (l^2 + (r - r_p)(r + r_p)) / (2 r), which avoids the 1 - cos(psi)
// cancellation of the reference's formula; each tesseroid's sum returns to
// FP64 for the accumulation.  The FP64 pipe, 1/64 of the FP32 rate on this
// GPU, then does almost nothing on the common path.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <string>

#include "../../include/harmonica_gb300.h"
#include "lean_packed.cuh"

namespace hg {

int set_error(int code, const std::string& msg);
int cuda_check(cudaError_t e, const char* what);

namespace tess {

constexpr int kThreads = 128;
constexpr int kWarps = kThreads / 32;
constexpr int kTile = 64;
constexpr int kSms = 152;
constexpr int kStackSize = 100;      // STACK_SIZE, tesseroid_gravity.py:27 (the largest allowed)
constexpr int64_t kMaxLeaves = 100000;  // MAX_DISCRETIZATIONS, tesseroid_gravity.py:28 (default)
constexpr int kNearCap = 64;         // split pairs buffered per warp
constexpr double kG = 6.6743e-11;    // choclo.constants.GRAVITATIONAL_CONST
constexpr double kDeg = 3.141592653589793 / 180.0;  // numpy.radians factor
constexpr double kPreTest = 1.0 + 0x1p-40;

// Rows of the prepared tesseroid records (structure of arrays, `stride`
// doubles per row).  Rows from kLonC on are staged in shared memory.
enum Row : int {
  kW, kE, kS, kN, kBot, kTop,
  kRho,       // density at the radial nodes k = 0 and 1 (equal for a constant
  kRho1,      // density; a density function evaluated at the node radii)
  kLonC,      // centre longitude (radians)
  kCosC,      // cos / sin of the centre latitude
  kSinC,
  kRC,        // centre radius
  kLLon,      // sizes (_tesseroid_dimensions)
  kLLat,
  kLRad,
  kSkip,      // 1: null tesseroid (zero size or density)
  // float2 rows (two floats in one 8-byte slot):
  kCentreXY,  // centre, Earth-centred Cartesian, FP32: (x, y)
  kCentreZ,   // (z, far_lon)
  kFar,       // (far_lat, far_rad): far = ratio * size * (1 + 2^-40) rounded up, +inf
              // when the size is not > 0
  kNodes,     // 24 rows: node (j, k) = jk, coordinate c: row kNodes + (jk * 3 + c) * 2
              // holds the high floats of nodes i = 0, 1, the next row the low floats
  kMasses = kNodes + 24,  // 8 rows: masses of nodes (jk, i = 0, 1), high then low floats
  kNodeR = kMasses + 8,   // 2 rows: node radii (k = 0, 1), high then low floats
  kRows = kNodeR + 2
};
constexpr int kSmemRows = kRows - kLonC;

struct GlqRule {
  double node[6];    // unscaled nodes: lon[2], lat[2], rad[2]
  double weight[6];  // weights in the same order
};

// Parameters of the adaptive discretisation.
struct Adapt {
  double ratio;        // DISTANCE_SIZE_RATII of the field
  int radial;          // split along the radius too
  int stack_size;      // <= kStackSize
  int64_t max_leaves;  // MAX_DISCRETIZATIONS
};

struct Station {
  double lon;   // radians
  double cphi;  // cos / sin of the latitude
  double sphi;
  double r;
};

using lean::F2;
using lean::P2;

// The point in Earth-centred Cartesian coordinates as float pairs, and 1 / r.
struct StationXYZ {
  F2 x, y, z;
  F2 r, inv_r;
  float r_f;
};

__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double rad(double deg) { return mul(deg, kDeg); }

// distance_spherical_core (utils.py:164-201).
__device__ __forceinline__ double distance_core(const Station& p, double lon_p, double cphi_p,
                                                double sphi_p, double r_p, double& cospsi) {
  const double coslambda = cos(sub(lon_p, p.lon));
  cospsi = add(mul(sphi_p, p.sphi), mul(mul(cphi_p, p.cphi), coslambda));
  const double dr = sub(p.r, r_p);
  return sqrt(add(mul(dr, dr), mul(mul(mul(2.0, p.r), r_p), sub(1.0, cospsi))));
}

// _tesseroid_dimensions (_tesseroid_utils.py:266-280).
__device__ __forceinline__ void dimensions(const double* t, double& l_lon, double& l_lat,
                                           double& l_rad) {
  const double w = rad(t[0]), e = rad(t[1]), s = rad(t[2]), n = rad(t[3]);
  const double top = t[5];
  const double latc = mul(add(n, s), 0.5);
  double sn, cn, ss, cs, sl, cl;
  sincos(n, &sn, &cn);
  sincos(s, &ss, &cs);
  sincos(latc, &sl, &cl);
  l_lat = mul(top, acos(add(mul(sn, ss), mul(cn, cs))));
  l_lon = mul(top, acos(add(mul(sl, sl), mul(mul(cl, cl), cos(sub(e, w))))));
  l_rad = sub(top, t[4]);
}

// Centre of a tesseroid as distance_spherical sees it (_tesseroid_utils.py:283-295).
__device__ __forceinline__ void centre(const double* t, double& lon_c, double& cos_c,
                                       double& sin_c, double& r_c) {
  lon_c = rad(mul(add(t[0], t[1]), 0.5));
  sincos(rad(mul(add(t[2], t[3]), 0.5)), &sin_c, &cos_c);
  r_c = mul(add(t[4], t[5]), 0.5);
}

// Point masses of gauss_legendre_quadrature (_tesseroid_utils.py:69-115).
struct Nodes {
  double lon[2], cphi[2], sphi[2], r[2], mass[8];
};

// density[k]: the density at radial node k (gauss_legendre_quadrature uses one
// value; gauss_legendre_quadrature_variable_density, _tesseroid_variable_
// density.py:18-107, the density function at radius_p of node k).
__device__ __forceinline__ void glq_nodes(const double* t, const double* density,
                                          const GlqRule& q, Nodes& nd) {
  const double w = t[0], e = t[1], s = t[2], n = t[3], bottom = t[4], top = t[5];
  const double a_factor =
      mul(mul(mul(0.125, rad(sub(e, w))), rad(sub(n, s))), sub(top, bottom));
#pragma unroll
  for (int j = 0; j < 2; j++) {
    const double lat_p = rad(add(mul(mul(0.5, sub(n, s)), q.node[2 + j]), mul(0.5, add(n, s))));
    sincos(lat_p, &nd.sphi[j], &nd.cphi[j]);
  }
#pragma unroll
  for (int k = 0; k < 2; k++)
    nd.r[k] = add(mul(mul(0.5, sub(top, bottom)), q.node[4 + k]), mul(0.5, add(top, bottom)));
#pragma unroll
  for (int i = 0; i < 2; i++)
    nd.lon[i] = rad(add(mul(mul(0.5, sub(e, w)), q.node[i]), mul(0.5, add(e, w))));
#pragma unroll
  for (int j = 0; j < 2; j++)
#pragma unroll
    for (int k = 0; k < 2; k++) {
      const double kappa = mul(mul(nd.r[k], nd.r[k]), nd.cphi[j]);
#pragma unroll
      for (int i = 0; i < 2; i++)
        nd.mass[(j * 2 + k) * 2 + i] =
            mul(mul(mul(mul(mul(density[k], a_factor), kappa), q.weight[i]), q.weight[2 + j]),
                q.weight[4 + k]);
    }
}

// distance / size < ratio, exactly as the reference evaluates it.
__device__ __forceinline__ bool split_axis(double d, double size, double ratio) {
  return d / size < ratio;
}

__device__ __forceinline__ P2 p2_of(const double* row_h, const double* row_l) {
  return P2{*reinterpret_cast<const float2*>(row_h), *reinterpret_cast<const float2*>(row_l)};
}

// Node sources for glq_sum_pairs: node (j, k) = jk of both longitudes as
// float pairs (lanes i = 0, 1) -- Cartesian coordinates and masses.
struct SmemNodes {  // prepared records staged in shared memory
  const double (*rows)[kTile];
  int col;
  __device__ __forceinline__ P2 radii() const {
    return p2_of(&rows[kNodeR - kLonC][col], &rows[kNodeR + 1 - kLonC][col]);
  }
  __device__ __forceinline__ void get(int jk, P2& x, P2& y, P2& z, P2& m) const {
    const int r0 = kNodes - kLonC + jk * 6;
    x = p2_of(&rows[r0][col], &rows[r0 + 1][col]);
    y = p2_of(&rows[r0 + 2][col], &rows[r0 + 3][col]);
    z = p2_of(&rows[r0 + 4][col], &rows[r0 + 5][col]);
    const int rm = kMasses - kLonC + jk * 2;
    m = p2_of(&rows[rm][col], &rows[rm + 1][col]);
  }
};

struct RegNodes {  // computed per small tesseroid of a split pair (thread-local)
  P2 x[4], y[4], z[4], m[4], r;
  __device__ __forceinline__ P2 radii() const { return r; }
  __device__ __forceinline__ void get(int jk, P2& xo, P2& yo, P2& zo, P2& mo) const {
    xo = x[jk];
    yo = y[jk];
    zo = z[jk];
    mo = m[jk];
  }
};

// The 8 point masses of one tesseroid at one point, on float pairs two
// nodes at a time (the lanes hold the nodes of the two longitudes):
// l^2 = |P - Q|^2 from the Cartesian difference (no 1 - cos(psi)
// cancellation), 1 / l by p2_rsqrt, and for g_z the radial component
// r - r_p cos(psi) = P . (P - Q) / r = (l^2 + (r - r_p)(r + r_p)) / (2 r).
// The point masses of gauss_legendre_quadrature with the kernels
// potential_spherical / gravity_u_spherical (point.py:323-354).  Each term's
// relative error is the 48-bit rounding of Earth-centred coordinates,
// ~2^-48 x 6.4e6 m / l, plus a few 2^-46: measured at most 2e-13 for l of
// 30 km - 3000 km (tests/test_float_pairs.py); the reference's own terms
// carry the rounding of 1 - cos(psi), ~2^-53 x 2 r r_p / l^2, which is
// larger for l below ~1000 km.  UNROLL: loop unrolling (1 keeps the code
// small).
template <int FIELD, int UNROLL, class Src>
__device__ __forceinline__ double glq_sum_pairs(const StationXYZ& q, const Src& src) {
  using namespace lean;
  const P2 px{sp2(q.x.h), sp2(q.x.l)}, py{sp2(q.y.h), sp2(q.y.l)}, pz{sp2(q.z.h), sp2(q.z.l)};
  // (r - r_k)(r + r_k) for the two node radii, lanes k = 0, 1
  P2 rr{sp2(0.0f), sp2(0.0f)};
  if (FIELD != 0) {
    const P2 pr{sp2(q.r.h), sp2(q.r.l)}, rk = src.radii();
    const P2 dif = p2_diff(pr, rk);
    const P2 sum_r = p2_diff(pr, p2_neg(rk));
    rr = p2_mul(dif, sum_r);
  }
  P2 sum{sp2(0.0f), sp2(0.0f)};
#pragma unroll UNROLL
  for (int jk = 0; jk < 4; jk++) {
    P2 nx, ny, nz, m;
    src.get(jk, nx, ny, nz, m);
    const P2 l2 = p2_norm2(p2_diff(px, nx), p2_diff(py, ny), p2_diff(pz, nz));
    const P2 inv = p2_rsqrt(l2);
    P2 term;
    if (FIELD == 0) {
      term = p2_mul(m, inv);
    } else {
      const int k = jk & 1;
      const P2 rrk{sp2(k ? rr.h.y : rr.h.x), sp2(k ? rr.l.y : rr.l.x)};
      const P2 pd2 = p2_add(l2, rrk);  // 2 r (r - r_p cos(psi))
      term = p2_mul(p2_mul(m, pd2), p2_mul(p2_mul(inv, inv), inv));
    }
    // running sum: two-sum of the high parts, low parts gathered unnormalised
    const P2 t = two_sum2(sum.h, term.h);
    sum = P2{t.h, add2(sum.l, add2(t.l, term.l))};
  }
  F2 s = f2_add(F2{sum.h.x, sum.l.x}, F2{sum.h.y, sum.l.y});
  if (FIELD != 0) s = f2_mul(s, q.inv_r);
  // G, the sign of gravity_u_spherical and the 1/2 of pd2, once per tesseroid
  return f2_to_double(s, 0) * (FIELD == 0 ? kG : -0.5 * kG);
}

// Cartesian float-pair nodes of gauss_legendre_quadrature's point masses.
__device__ __forceinline__ void cartesian_nodes(const Nodes& nd, lean::F2 (*xyz)[3][2],
                                                lean::F2 (*m)[2], lean::F2* r) {
  r[0] = lean::double_to_f2(nd.r[0]);
  r[1] = lean::double_to_f2(nd.r[1]);
  double c_lon[2], s_lon[2];
#pragma unroll
  for (int i = 0; i < 2; i++) sincos(nd.lon[i], &s_lon[i], &c_lon[i]);
#pragma unroll
  for (int jj = 0; jj < 2; jj++)
#pragma unroll
    for (int k = 0; k < 2; k++) {
      const int jk = jj * 2 + k;
      const double rc = nd.r[k] * nd.cphi[jj];
#pragma unroll
      for (int i = 0; i < 2; i++) {
        xyz[jk][0][i] = lean::double_to_f2(rc * c_lon[i]);
        xyz[jk][1][i] = lean::double_to_f2(rc * s_lon[i]);
        xyz[jk][2][i] = lean::double_to_f2(nd.r[k] * nd.sphi[jj]);
        m[jk][i] = lean::double_to_f2(nd.mass[jk * 2 + i]);
      }
    }
}

// A small tesseroid of a split pair: its point masses (the reference's
// positions and masses) summed on float pairs.
template <int FIELD>
__device__ __forceinline__ double glq_leaf_pairs(const StationXYZ& q3, const Nodes& nd) {
  lean::F2 xyz[4][3][2], m[4][2], r[2];
  cartesian_nodes(nd, xyz, m, r);
  RegNodes src;
  src.r = lean::pk(r[0], r[1]);
#pragma unroll
  for (int jk = 0; jk < 4; jk++) {
    src.x[jk] = lean::pk(xyz[jk][0][0], xyz[jk][0][1]);
    src.y[jk] = lean::pk(xyz[jk][1][0], xyz[jk][1][1]);
    src.z[jk] = lean::pk(xyz[jk][2][0], xyz[jk][2][1]);
    src.m[jk] = lean::pk(m[jk][0], m[jk][1]);
  }
  return glq_sum_pairs<FIELD, 1>(q3, src);
}

// _adaptive_discretization (_tesseroid_utils.py:150-241) for one pair, each
// small tesseroid integrated when popped (the order in which the reference
// stores and then integrates them).  status: 1 stack overflow, 2 more than
// MAX_DISCRETIZATIONS small tesseroids.
template <int FIELD>
__device__ __noinline__ double adaptive_pair(const Station& p, const StationXYZ& q3,
                                             const double* root, const double* density,
                                             const Adapt& ad,
                                             const GlqRule& q, int& status) {
  double stack[kStackSize][6];
#pragma unroll
  for (int c = 0; c < 6; c++) stack[0][c] = root[c];
  const double ratio = ad.ratio;
  const bool radial = ad.radial != 0;
  int top = 0;
  int64_t leaves = 0;
  double acc = 0.0;
  while (top >= 0) {
    double t[6];
#pragma unroll
    for (int c = 0; c < 6; c++) t[c] = stack[top][c];
    top--;
    double l_lon, l_lat, l_rad;
    dimensions(t, l_lon, l_lat, l_rad);
    double lon_c, cos_c, sin_c, r_c, cospsi;
    centre(t, lon_c, cos_c, sin_c, r_c);
    const double d = distance_core(p, lon_c, cos_c, sin_c, r_c, cospsi);
    const int n_lon = d / l_lon < ratio ? 2 : 1;
    const int n_lat = d / l_lat < ratio ? 2 : 1;
    const int n_rad = (d / l_rad < ratio && radial) ? 2 : 1;
    const int n_child = n_lon * n_lat * n_rad;
    if (n_child > 1) {
      if ((top + 1) + n_child > ad.stack_size) {
        status |= 1;
        return acc;
      }
      const double d_lon = sub(t[1], t[0]) / n_lon;
      const double d_lat = sub(t[3], t[2]) / n_lat;
      const double d_rad = sub(t[5], t[4]) / n_rad;
      for (int i = 0; i < n_lon; i++)
        for (int j = 0; j < n_lat; j++)
          for (int k = 0; k < n_rad; k++) {
            top++;
            stack[top][0] = add(t[0], mul(d_lon, (double)i));
            stack[top][1] = add(t[0], mul(d_lon, (double)(i + 1)));
            stack[top][2] = add(t[2], mul(d_lat, (double)j));
            stack[top][3] = add(t[2], mul(d_lat, (double)(j + 1)));
            stack[top][4] = add(t[4], mul(d_rad, (double)k));
            stack[top][5] = add(t[4], mul(d_rad, (double)(k + 1)));
          }
    } else {
      if (leaves + 1 > ad.max_leaves) {
        status |= 2;
        return acc;
      }
      leaves++;
      Nodes nd;
      glq_nodes(t, density, q, nd);
      acc += glq_leaf_pairs<FIELD>(q3, nd);
    }
  }
  return acc;
}

__global__ void prepare_kernel(const double* __restrict__ aos, const double* __restrict__ density,
                               int per_node, int64_t m, double* __restrict__ rec, int64_t stride,
                               double ratio, GlqRule q) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= m) return;
  double t[6];
#pragma unroll
  for (int c = 0; c < 6; c++) t[c] = aos[6 * j + c];
  double rho[2];
  rho[0] = per_node ? density[2 * j] : density[j];
  rho[1] = per_node ? density[2 * j + 1] : rho[0];
#pragma unroll
  for (int c = 0; c < 6; c++) rec[c * stride + j] = t[c];
  rec[kRho * stride + j] = rho[0];
  rec[kRho1 * stride + j] = rho[1];
  // _discard_null_tesseroids (_tesseroid_utils.py:503-538); a tesseroid with a
  // NaN or infinite bound or density that is not null makes the reference's
  // result NaN: flag 2
  const bool null =
      t[0] == t[1] || t[2] == t[3] || t[4] == t[5] || (rho[0] == 0.0 && rho[1] == 0.0);
  bool finite = isfinite(rho[0]) && isfinite(rho[1]);
#pragma unroll
  for (int c = 0; c < 6; c++) finite = finite && isfinite(t[c]);
  rec[kSkip * stride + j] = null ? 1.0 : (finite ? 0.0 : 2.0);
  double l[3];
  dimensions(t, l[0], l[1], l[2]);
  double lon_c, cos_c, sin_c, r_c;
  centre(t, lon_c, cos_c, sin_c, r_c);
  rec[kLonC * stride + j] = lon_c;
  rec[kCosC * stride + j] = cos_c;
  rec[kSinC * stride + j] = sin_c;
  rec[kRC * stride + j] = r_c;
  float far[3];
#pragma unroll
  for (int a = 0; a < 3; a++) {
    rec[(kLLon + a) * stride + j] = l[a];
    far[a] = l[a] > 0.0 ? __double2float_ru(mul(mul(ratio, l[a]), kPreTest)) : INFINITY;
  }
  double s_lon_c, c_lon_c;
  sincos(lon_c, &s_lon_c, &c_lon_c);
  const double rcc = r_c * cos_c;
  float2* f2row = reinterpret_cast<float2*>(rec);
  f2row[kCentreXY * stride + j] = make_float2((float)(rcc * c_lon_c), (float)(rcc * s_lon_c));
  f2row[kCentreZ * stride + j] = make_float2((float)(r_c * sin_c), far[0]);
  f2row[kFar * stride + j] = make_float2(far[1], far[2]);
  Nodes nd;
  glq_nodes(t, rho, q, nd);
  lean::F2 xyz[4][3][2], mass[4][2], nr[2];
  cartesian_nodes(nd, xyz, mass, nr);
  f2row[kNodeR * stride + j] = make_float2(nr[0].h, nr[1].h);
  f2row[(kNodeR + 1) * stride + j] = make_float2(nr[0].l, nr[1].l);
#pragma unroll
  for (int jk = 0; jk < 4; jk++) {
#pragma unroll
    for (int c = 0; c < 3; c++) {
      f2row[(kNodes + (jk * 3 + c) * 2) * stride + j] =
          make_float2(xyz[jk][c][0].h, xyz[jk][c][1].h);
      f2row[(kNodes + (jk * 3 + c) * 2 + 1) * stride + j] =
          make_float2(xyz[jk][c][0].l, xyz[jk][c][1].l);
    }
    f2row[(kMasses + jk * 2) * stride + j] = make_float2(mass[jk][0].h, mass[jk][1].h);
    f2row[(kMasses + jk * 2 + 1) * stride + j] = make_float2(mass[jk][0].l, mass[jk][1].l);
  }
}

// A point's data for the lane that runs one of its split pairs.
struct StationSh {
  Station p;
  StationXYZ q;
};

// Split pair `ent` of a chunk's list: (tesseroid index in the chunk) << 5 | lane.
template <int FIELD>
__device__ __forceinline__ double run_entry(uint32_t ent, const StationSh& st,
                                            const double* __restrict__ rec, int64_t stride,
                                            int64_t p0, const Adapt& ad, const GlqRule& q,
                                            int& status) {
  const int64_t j = p0 + (int64_t)(ent >> 5);
  double root[6];
#pragma unroll
  for (int c = 0; c < 6; c++) root[c] = rec[c * stride + j];
  const double rho[2] = {rec[kRho * stride + j], rec[kRho1 * stride + j]};
  return adaptive_pair<FIELD>(st.p, st.q, root, rho, ad, q, status);
}

// A warp's list is full: run it, 32 pairs at a time (one per lane), and add
// each result to its point's sum in list order.
template <int FIELD>
__device__ __forceinline__ void flush_warp(const uint32_t* list, int count, int lane,
                                           const StationSh* warp_st,
                                           const double* __restrict__ rec, int64_t stride,
                                           int64_t p0, const Adapt& ad, const GlqRule& q,
                                           double& acc, int& status) {
  for (int r0 = 0; r0 < count; r0 += 32) {
    const int e = r0 + lane;
    const bool has = e < count;
    const uint32_t ent = has ? list[e] : 0u;
    const int owner = has ? (int)(ent & 31u) : lane;
    double contrib = 0.0;
    if (has) contrib = run_entry<FIELD>(ent, warp_st[owner], rec, stride, p0, ad, q, status);
    __syncwarp();
    const int n = min(32, count - r0);
    for (int k = 0; k < n; k++) {
      const double v = __shfl_sync(0xffffffffu, contrib, k);
      const int o = __shfl_sync(0xffffffffu, owner, k);
      if (lane == o) acc += v;
    }
  }
  __syncwarp();
}

// Per point, once per launch: the reference's radians, cos/sin of the
// latitude and radius, and the Cartesian float pairs of the fast path.
__global__ void stations_kernel(const double* __restrict__ lon_deg,
                                const double* __restrict__ lat_deg,
                                const double* __restrict__ radius, int64_t n_obs,
                                StationSh* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_obs) return;
  Station p;
  p.lon = rad(lon_deg[i]);
  sincos(rad(lat_deg[i]), &p.sphi, &p.cphi);
  p.r = radius[i];
  StationXYZ q3;
  double slon, clon;
  sincos(p.lon, &slon, &clon);
  const double rc = p.r * p.cphi;
  q3.x = lean::double_to_f2(rc * clon);
  q3.y = lean::double_to_f2(rc * slon);
  q3.z = lean::double_to_f2(p.r * p.sphi);
  q3.r = lean::double_to_f2(p.r);
  q3.inv_r = lean::double_to_f2(1.0 / p.r);
  q3.r_f = (float)p.r;
  out[i] = StationSh{p, q3};
}

template <int FIELD>
__global__ void __launch_bounds__(kThreads, 4) forward_kernel(
    const StationSh* __restrict__ stations, int64_t n_obs, const double* __restrict__ rec,
    int64_t stride, int64_t n_tess, int64_t chunk, Adapt ad, GlqRule q,
    double* __restrict__ dst, int64_t dst_chunk_stride, double out_scale,
    int32_t* __restrict__ status_out) {
  __shared__ double sh[kSmemRows][kTile];
  __shared__ uint32_t near_list[kWarps][kNearCap];
  __shared__ int near_count[kWarps];
  __shared__ double contrib[kWarps * kNearCap];
  __shared__ StationSh st[kThreads];
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int64_t i = (int64_t)blockIdx.x * kThreads + threadIdx.x;
  const bool active = i < n_obs;
  const StationSh me = stations[active ? i : 0];
  const Station p = me.p;
  const StationXYZ q3 = me.q;
  st[threadIdx.x] = me;  // read after the first barrier below
  const bool rad_split = ad.radial != 0;
  const double ratio = ad.ratio;

  double acc = 0.0;
  int status = 0;
  int n_near = 0;  // warp-uniform
  const int64_t p0 = (int64_t)blockIdx.y * chunk;
  const int64_t p1 = min(p0 + chunk, n_tess);
  for (int64_t base = p0; base < p1; base += kTile) {
    const int cnt = (int)min((int64_t)kTile, p1 - base);
    __syncthreads();
    for (int idx = threadIdx.x; idx < kSmemRows * kTile; idx += kThreads) {
      const int r = idx / kTile, c = idx % kTile;
      sh[r][c] = c < cnt ? rec[(int64_t)(kLonC + r) * stride + base + c] : 0.0;
    }
    __syncthreads();
    for (int c = 0; c < cnt; c++) {
      const double skip = sh[kSkip - kLonC][c];  // same for the whole block
      if (skip != 0.0) {
        if (skip == 2.0) acc += NAN;
        continue;
      }
      bool near = false;
      if (active) {
#define S(row) sh[(row) - kLonC][c]
#define F(row) (*reinterpret_cast<const float2*>(&sh[(row) - kLonC][c]))
        // FP32 distance to the centre in Cartesian coordinates.  Its error
        // against the reference's distance is below 2^-22 (r + r_c) from the
        // coordinates' rounding, ~0.1 m from the reference's own rounding at
        // d >= 1 m and 2^-21 relative from the arithmetic, so
        // d2 (1 - 2^-19) >= (far + 2^-21 (r + r_c) + 1 m)^2 proves
        // distance / size >= ratio on that axis.
        const float2 cxy = F(kCentreXY), cz = F(kCentreZ), fl = F(kFar);
        const float ddx = q3.x.h - cxy.x, ddy = q3.y.h - cxy.y, ddz = q3.z.h - cz.x;
        const float d2 = fmaf(ddx, ddx, fmaf(ddy, ddy, ddz * ddz)) * (1.0f - 0x1p-19f);
        const float slack = fmaf(0x1p-21f, q3.r_f + (float)S(kRC), 1.0f);
        const float t_lon = cz.y + slack, t_lat = fl.x + slack, t_rad = fl.y + slack;
        if (!(d2 >= t_lon * t_lon) || !(d2 >= t_lat * t_lat) ||
            (rad_split && !(d2 >= t_rad * t_rad))) {
          // undecided: the reference's distance and quotients
          double cospsi;
          const double d = distance_core(p, S(kLonC), S(kCosC), S(kSinC), S(kRC), cospsi);
          near = split_axis(d, S(kLLon), ratio) || split_axis(d, S(kLLat), ratio) ||
                 (rad_split && split_axis(d, S(kLRad), ratio));
        }
        if (!near) acc += glq_sum_pairs<FIELD, 4>(q3, SmemNodes{sh, c});
#undef F
#undef S
      }
      const unsigned ball = __ballot_sync(0xffffffffu, near);
      if (ball) {
        const int add_n = __popc(ball);
        if (n_near + add_n > kNearCap) {
          flush_warp<FIELD>(near_list[warp], n_near, lane, &st[warp * 32], rec, stride, p0, ad,
                            q, acc, status);
          n_near = 0;
        }
        if (near)
          near_list[warp][n_near + __popc(ball & ((1u << lane) - 1u))] =
              ((uint32_t)(base + c - p0) << 5) | (uint32_t)lane;
        n_near += add_n;
        __syncwarp();
      }
    }
  }
  // the split pairs left in the four lists run on all the block's lanes
  // together; each point then adds its results in its list's order
  if (lane == 0) near_count[warp] = n_near;
  __syncthreads();
  int offs[kWarps], total = 0;
#pragma unroll
  for (int w = 0; w < kWarps; w++) {
    offs[w] = total;
    total += near_count[w];
  }
  for (int e = threadIdx.x; e < total; e += kThreads) {
    int w = 0;
#pragma unroll
    for (int v = 1; v < kWarps; v++) w += e >= offs[v] ? 1 : 0;
    const uint32_t ent = near_list[w][e - offs[w]];
    contrib[e] = run_entry<FIELD>(ent, st[w * 32 + (int)(ent & 31u)], rec, stride, p0, ad, q,
                                  status);
  }
  __syncthreads();
  for (int k = 0; k < n_near; k++)
    if ((int)(near_list[warp][k] & 31u) == lane) acc += contrib[offs[warp] + k];
  if (status && status_out) atomicOr(status_out, status);
  if (active) dst[(int64_t)blockIdx.y * dst_chunk_stride + i] = mul(acc, out_scale);
}

// Sum of the chunk partials of 32 points per block: thread (x, y) adds the
// chunks y, y + 16, ... of point x (coalesced rows), then the 16 group sums
// are added in order of y.  Fixed order for a given number of chunks:
// deterministic.
constexpr int kReduceGroups = 16;

__global__ void __launch_bounds__(32 * kReduceGroups) reduce_kernel(
    const double* __restrict__ part, int64_t n_chunks, int64_t n_obs, double scale,
    double* __restrict__ out) {
  __shared__ double group[kReduceGroups][32];
  const int64_t i = (int64_t)blockIdx.x * 32 + threadIdx.x;
  double s = 0.0;
  if (i < n_obs)
    for (int64_t c = threadIdx.y; c < n_chunks; c += kReduceGroups) s += part[c * n_obs + i];
  group[threadIdx.y][threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.y == 0 && i < n_obs) {
    double t = 0.0;
#pragma unroll
    for (int g = 0; g < kReduceGroups; g++) t += group[g][threadIdx.x];
    out[i] = mul(t, scale);
  }
}

// Python's float modulo (x % 360, result in [0, 360)).
__device__ __forceinline__ double py_mod360(double x) {
  double m = fmod(x, 360.0);
  if (m != 0.0) {
    if (m < 0.0) m = add(m, 360.0);
  } else {
    m = 0.0;
  }
  return m;
}

// _check_points_outside_tesseroids (_tesseroid_utils.py:446-468).
__global__ void __launch_bounds__(kThreads) inside_kernel(
    const double* __restrict__ lon, const double* __restrict__ lat,
    const double* __restrict__ radius, int64_t n_obs, const double* __restrict__ aos, int64_t m,
    int64_t chunk, long long* __restrict__ conflicts, int64_t cap,
    unsigned long long* __restrict__ count) {
  __shared__ double sh[6][kTile];
  __shared__ double bound[4];  // tile: lowest bottom, highest top, lowest south, highest north
  const int64_t i = (int64_t)blockIdx.x * kThreads + threadIdx.x;
  const bool active = i < n_obs;
  const double lo = active ? lon[i] : 0.0;
  const double la = active ? lat[i] : 0.0;
  const double r = active ? radius[i] : 0.0;
  const double lon_360 = py_mod360(lo);
  const double lon_180 = sub(py_mod360(add(lo, 180.0)), 180.0);
  const int64_t p0 = (int64_t)blockIdx.y * chunk;
  const int64_t p1 = min(p0 + chunk, m);
  for (int64_t base = p0; base < p1; base += kTile) {
    const int cnt = (int)min((int64_t)kTile, p1 - base);
    __syncthreads();
    for (int idx = threadIdx.x; idx < 6 * kTile; idx += kThreads) {
      const int c = idx / 6, k = idx % 6;
      if (c < cnt) sh[k][c] = aos[6 * (base + c) + k];
    }
    __syncthreads();
    if (threadIdx.x < 32) {
      // the tile's radial and latitudinal extent (fmin/fmax skip NaN bounds,
      // whose tesseroids contain no point)
      double lo_b = INFINITY, hi_t = -INFINITY, lo_s = INFINITY, hi_n = -INFINITY;
      for (int c = threadIdx.x; c < cnt; c += 32) {
        lo_b = fmin(lo_b, sh[4][c]);
        hi_t = fmax(hi_t, sh[5][c]);
        lo_s = fmin(lo_s, sh[2][c]);
        hi_n = fmax(hi_n, sh[3][c]);
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        lo_b = fmin(lo_b, __shfl_xor_sync(0xffffffffu, lo_b, o));
        hi_t = fmax(hi_t, __shfl_xor_sync(0xffffffffu, hi_t, o));
        lo_s = fmin(lo_s, __shfl_xor_sync(0xffffffffu, lo_s, o));
        hi_n = fmax(hi_n, __shfl_xor_sync(0xffffffffu, hi_n, o));
      }
      if (threadIdx.x == 0) {
        bound[0] = lo_b;
        bound[1] = hi_t;
        bound[2] = lo_s;
        bound[3] = hi_n;
      }
    }
    __syncthreads();
    if (!active) continue;
    // a point outside the tile's extent is in none of its tesseroids (points
    // above a layer skip every tile)
    if (!(bound[0] < r && r < bound[1] && bound[2] < la && la < bound[3])) continue;
    for (int c = 0; c < cnt; c++) {
      const double w = sh[0][c], e = sh[1][c], s = sh[2][c], n = sh[3][c];
      const double b = sh[4][c], t = sh[5][c];
      const bool in_lon = (w < lon_180 && lon_180 < e) || (w < lon_360 && lon_360 < e);
      if (in_lon && s < la && la < n && b < r && r < t) {
        const unsigned long long k = atomicAdd(count, 1ull);
        if ((int64_t)k < cap) {
          conflicts[2 * k] = (long long)i;
          conflicts[2 * k + 1] = (long long)(base + c);
        }
      }
    }
  }
}

struct Plan {
  int64_t n_tiles, n_chunks, chunk;
  size_t rec_bytes, station_bytes, part_bytes;
};

Plan make_plan(int64_t n_obs, int64_t m) {
  Plan p;
  p.n_tiles = (n_obs + kThreads - 1) / kThreads;
  if (p.n_tiles < 1) p.n_tiles = 1;
  int64_t m_tiles = (m + kTile - 1) / kTile;
  if (m_tiles < 1) m_tiles = 1;
  // about 96 waves of 4 resident CTAs per SM (HG_TESS_WAVES overrides),
  // which on the layer workloads means one 64-tesseroid tile per CTA: the
  // split pairs, which cost ~100x an unsplit one, then spread over many
  // short CTAs instead of lengthening a few (measured on the 93,121-
  // tesseroid layer: 8 waves 2.2e10 pairs/s, 24 2.8e10, 96 3.1e10).  The
  // chunk partials stay below target x 128 points x 8 bytes (60 MB).
  static const int64_t waves = [] {
    const char* v = std::getenv("HG_TESS_WAVES");
    const long w = v ? std::strtol(v, nullptr, 10) : 96;
    return (int64_t)(w >= 1 && w <= 256 ? w : 96);
  }();
  const int64_t target = (int64_t)kSms * 4 * waves;
  int64_t want = (target + p.n_tiles - 1) / p.n_tiles;
  // the per-warp list keeps the index within the chunk in 27 bits
  const int64_t min_chunks = (m_tiles * kTile + (1ll << 26) - 1) >> 26;
  if (want < min_chunks) want = min_chunks;
  if (want > m_tiles) want = m_tiles;
  if (want > 65535) want = 65535;
  if (want < 1) want = 1;
  const int64_t tiles_per_chunk = (m_tiles + want - 1) / want;
  p.chunk = tiles_per_chunk * kTile;
  p.n_chunks = (m + p.chunk - 1) / p.chunk;
  if (p.n_chunks < 1) p.n_chunks = 1;
  p.rec_bytes = ((size_t)kRows * (size_t)(m > 0 ? m : 1) * sizeof(double) + 255) & ~(size_t)255;
  p.station_bytes = ((size_t)(n_obs > 0 ? n_obs : 1) * sizeof(StationSh) + 255) & ~(size_t)255;
  p.part_bytes = p.n_chunks > 1 ? (size_t)p.n_chunks * n_obs * sizeof(double) : 0;
  return p;
}

GlqRule make_rule(const double* nodes, const double* weights) {
  GlqRule q;
  const double x = 1.0 / std::sqrt(3.0);
  for (int a = 0; a < 3; a++) {
    q.node[2 * a] = nodes ? nodes[2 * a] : -x;
    q.node[2 * a + 1] = nodes ? nodes[2 * a + 1] : x;
    q.weight[2 * a] = weights ? weights[2 * a] : 1.0;
    q.weight[2 * a + 1] = weights ? weights[2 * a + 1] : 1.0;
  }
  return q;
}

}  // namespace tess
}  // namespace hg

using namespace hg;

extern "C" {

int hg_tesseroid_forward_workspace(int64_t n_obs, int64_t n_tesseroids, size_t* bytes) {
  if (!bytes) return set_error(HG_ERR_INVALID, "null pointer");
  if (n_obs < 0 || n_tesseroids < 0) return set_error(HG_ERR_INVALID, "bad sizes");
  const tess::Plan p = tess::make_plan(n_obs, n_tesseroids);
  *bytes = p.rec_bytes + p.station_bytes + p.part_bytes;
  return HG_OK;
}

int hg_tesseroid_forward(const double* longitude, const double* latitude, const double* radius,
                         int64_t n_obs, const double* tesseroids, const double* density,
                         int32_t density_per_node, int64_t n_tesseroids, int32_t field,
                         int32_t radial_discretization,
                         int32_t stack_size, int64_t max_discretizations,
                         const double* glq_nodes, const double* glq_weights, double* out,
                         int32_t* status, void* workspace, size_t workspace_bytes,
                         void* stream) {
  if (n_obs < 0 || n_tesseroids < 0) return set_error(HG_ERR_INVALID, "bad sizes");
  if (stack_size > tess::kStackSize)
    return set_error(HG_ERR_INVALID, "tesseroid stack size above 100 is not supported");
  if (field != 0 && field != 3)
    return set_error(HG_ERR_INVALID, "tesseroid field must be 0 (potential) or 3 (g_z)");
  if (n_obs == 0) return HG_OK;
  if (!longitude || !latitude || !radius || !out) return set_error(HG_ERR_INVALID, "null pointer");
  if (n_tesseroids > 0 && (!tesseroids || !density))
    return set_error(HG_ERR_INVALID, "null tesseroid pointer");
  cudaStream_t st = (cudaStream_t)stream;
  const double scale = field == 3 ? -1e5 : 1.0;  // tesseroid_gravity.py:209-215
  if (n_tesseroids == 0)
    return cuda_check(cudaMemsetAsync(out, 0, sizeof(double) * n_obs, st), "cudaMemsetAsync");
  const tess::Plan plan = tess::make_plan(n_obs, n_tesseroids);
  if (plan.n_tiles > 2147483647LL) return set_error(HG_ERR_INVALID, "too many points");
  const size_t need = plan.rec_bytes + plan.station_bytes + plan.part_bytes;
  bool own = false;
  if (workspace == nullptr) {
    cudaError_t e = cudaMallocAsync(&workspace, need, st);
    if (e != cudaSuccess) return cuda_check(e, "cudaMallocAsync(workspace)");
    own = true;
  } else if (workspace_bytes < need) {
    return set_error(HG_ERR_INVALID, "workspace too small");
  }
  double* rec = static_cast<double*>(workspace);
  tess::StationSh* stations =
      reinterpret_cast<tess::StationSh*>(static_cast<char*>(workspace) + plan.rec_bytes);
  double* part = reinterpret_cast<double*>(static_cast<char*>(workspace) + plan.rec_bytes +
                                           plan.station_bytes);
  const tess::GlqRule q = tess::make_rule(glq_nodes, glq_weights);
  tess::Adapt ad;
  ad.ratio = field == 3 ? 2.5 : 1.0;  // DISTANCE_SIZE_RATII, tesseroid_gravity.py:30
  ad.radial = radial_discretization ? 1 : 0;
  ad.stack_size = stack_size > 0 ? stack_size : tess::kStackSize;
  ad.max_leaves = max_discretizations > 0 ? max_discretizations : tess::kMaxLeaves;
  const int threads = 256;
  tess::prepare_kernel<<<(unsigned)((n_tesseroids + threads - 1) / threads), threads, 0, st>>>(
      tesseroids, density, density_per_node ? 1 : 0, n_tesseroids, rec, n_tesseroids, ad.ratio, q);
  int rc = cuda_check(cudaGetLastError(), "tesseroid prepare_kernel launch");
  if (rc == HG_OK) {
    tess::stations_kernel<<<(unsigned)((n_obs + threads - 1) / threads), threads, 0, st>>>(
        longitude, latitude, radius, n_obs, stations);
    rc = cuda_check(cudaGetLastError(), "tesseroid stations_kernel launch");
  }
  if (rc == HG_OK) {
    const bool direct = plan.n_chunks == 1;
    double* dst = direct ? out : part;
    const dim3 grid((unsigned)plan.n_tiles, (unsigned)plan.n_chunks);
    if (field == 0)
      tess::forward_kernel<0><<<grid, tess::kThreads, 0, st>>>(
          stations, n_obs, rec, n_tesseroids, n_tesseroids, plan.chunk, ad, q, dst, n_obs,
          direct ? scale : 1.0, status);
    else
      tess::forward_kernel<1><<<grid, tess::kThreads, 0, st>>>(
          stations, n_obs, rec, n_tesseroids, n_tesseroids, plan.chunk, ad, q, dst, n_obs,
          direct ? scale : 1.0, status);
    rc = cuda_check(cudaGetLastError(), "tesseroid forward_kernel launch");
    if (rc == HG_OK && !direct) {
      tess::reduce_kernel<<<(unsigned)((n_obs + 31) / 32), dim3(32, tess::kReduceGroups), 0,
                            st>>>(part, plan.n_chunks, n_obs, scale, out);
      rc = cuda_check(cudaGetLastError(), "tesseroid reduce_kernel launch");
    }
  }
  if (own) cudaFreeAsync(workspace, st);
  return rc;
}

int hg_tesseroid_inside(const double* longitude, const double* latitude, const double* radius,
                        int64_t n_obs, const double* tesseroids, int64_t n_tesseroids,
                        int64_t* conflicts, int64_t capacity, int64_t* n_conflicts,
                        void* stream) {
  if (n_obs < 0 || n_tesseroids < 0 || capacity < 0) return set_error(HG_ERR_INVALID, "bad sizes");
  if (!n_conflicts) return set_error(HG_ERR_INVALID, "null pointer");
  cudaStream_t st = (cudaStream_t)stream;
  int rc = cuda_check(cudaMemsetAsync(n_conflicts, 0, sizeof(int64_t), st), "cudaMemsetAsync");
  if (rc != HG_OK || n_obs == 0 || n_tesseroids == 0) return rc;
  if (!longitude || !latitude || !radius || !tesseroids || (capacity > 0 && !conflicts))
    return set_error(HG_ERR_INVALID, "null pointer");
  const tess::Plan plan = tess::make_plan(n_obs, n_tesseroids);
  const dim3 grid((unsigned)plan.n_tiles, (unsigned)plan.n_chunks);
  tess::inside_kernel<<<grid, tess::kThreads, 0, st>>>(
      longitude, latitude, radius, n_obs, tesseroids, n_tesseroids, plan.chunk,
      reinterpret_cast<long long*>(conflicts), capacity,
      reinterpret_cast<unsigned long long*>(n_conflicts));
  return cuda_check(cudaGetLastError(), "tesseroid inside_kernel launch");
}

}  // extern "C"
