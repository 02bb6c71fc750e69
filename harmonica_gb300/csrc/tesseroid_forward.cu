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
// Arithmetic.  FP64 throughout.  The split decisions and every small
// tesseroid of a split pair follow the reference's operation order without
// contraction into fused multiply-adds (__dmul_rn / __dadd_rn), so they
// differ from the reference only through the last bits of cos/sin/acos.  The
// split test distance / size < ratio is evaluated exactly whenever it is not
// settled by a pre-test on the squared distance with a rigorous error margin
// (distance >= ratio * size * (1 + 2^-40) proves "no split").  Unsplit
// tesseroids -- nearly all pairs -- are summed by glq_eval_fast: the same 8
// point masses with cos(lambda_p - lambda) from precomputed cosines and sines
// and 1 / l from a reciprocal square root, within a few units in the last
// place of the reference's terms at about half the FP64 instructions.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <string>

#include "../../include/harmonica_gb300.h"
#include "lean_math.cuh"

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
  kW, kE, kS, kN, kBot, kTop, kRho,
  kLonC,      // centre longitude (radians)
  kCosC,      // cos / sin of the centre latitude
  kSinC,
  kRC,        // centre radius
  kCosLonC,   // cos / sin of the centre longitude
  kSinLonC,
  kFar2Lon,   // (ratio * size * (1 + 2^-40))^2 when size > 0, else +inf
  kFar2Lat,
  kFar2Rad,
  kLLon,      // sizes (_tesseroid_dimensions)
  kLLat,
  kLRad,
  kNodeCosLon,                    // 2 rows: cos of node longitudes, i = 0, 1
  kNodeSinLon = kNodeCosLon + 2,  // 2 rows: sin of node longitudes
  kNodeCos = kNodeSinLon + 2,     // 2 rows: cos of node latitudes, j = 0, 1
  kNodeSin = kNodeCos + 2,  // 2 rows: sin of node latitudes
  kNodeRad = kNodeSin + 2,  // 2 rows: node radii, k = 0, 1
  kMass = kNodeRad + 2,     // 8 rows: masses, index (j * 2 + k) * 2 + i
  kSkip = kMass + 8,        // 1: null tesseroid (zero size or density)
  kRows
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
  double clon;  // cos / sin of the longitude
  double slon;
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

__device__ __forceinline__ void glq_nodes(const double* t, double density, const GlqRule& q,
                                          Nodes& nd) {
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
            mul(mul(mul(mul(mul(density, a_factor), kappa), q.weight[i]), q.weight[2 + j]),
                q.weight[4 + k]);
    }
}

// Sum of the 8 point masses at one point (the loop of
// gauss_legendre_quadrature with potential_spherical / gravity_u_spherical,
// point.py:323-354).  FIELD 0: potential; 1: radial (upward) acceleration, SI.
template <int FIELD>
__device__ __forceinline__ double glq_eval(const Station& p, const double* lon_n,
                                           const double* cphi_n, const double* sphi_n,
                                           const double* r_n, const double* mass) {
  double coslambda[2];
#pragma unroll
  for (int i = 0; i < 2; i++) coslambda[i] = cos(sub(lon_n[i], p.lon));
  const double two_r = mul(2.0, p.r);
  double result = 0.0;
#pragma unroll
  for (int j = 0; j < 2; j++) {
    const double s_term = mul(sphi_n[j], p.sphi);
    const double c_term = mul(cphi_n[j], p.cphi);
#pragma unroll
    for (int k = 0; k < 2; k++) {
      const double dr = sub(p.r, r_n[k]);
      const double dr2 = mul(dr, dr);
      const double rr = mul(two_r, r_n[k]);
#pragma unroll
      for (int i = 0; i < 2; i++) {
        const double cospsi = add(s_term, mul(c_term, coslambda[i]));
        const double dist = sqrt(add(dr2, mul(rr, sub(1.0, cospsi))));
        double kern;
        if (FIELD == 0) {
          kern = mul(1.0 / dist, kG);
        } else {
          const double delta_z = sub(p.r, mul(r_n[k], cospsi));
          kern = mul(-kG, delta_z) / mul(mul(dist, dist), dist);
        }
        result = add(result, mul(mass[(j * 2 + k) * 2 + i], kern));
      }
    }
  }
  return result;
}

// distance / size < ratio, exactly as the reference evaluates it.
__device__ __forceinline__ bool split_axis(double d, double size, double ratio) {
  return d / size < ratio;
}

// The 8 point masses of an unsplit tesseroid at one point, rearranged for
// the FP64 pipe: cos(lambda_p - lambda) from the cosines and sines of both
// longitudes (cos a cos b + sin a sin b), and 1 / l from a reciprocal square
// root (FP32 seed, two FP64 Newton steps) instead of a square root and a
// division.  Same point masses and kernels as glq_eval; each term differs
// from it by a few units in the last place of cos(psi) and l.
template <int FIELD>
__device__ __forceinline__ double glq_eval_fast(const Station& p, const double* clon_n,
                                                const double* slon_n, const double* cphi_n,
                                                const double* sphi_n, const double* r_n,
                                                const double* mass) {
  double coslambda[2];
#pragma unroll
  for (int i = 0; i < 2; i++) coslambda[i] = fma(clon_n[i], p.clon, slon_n[i] * p.slon);
  const double two_r = 2.0 * p.r;
  double result = 0.0;
#pragma unroll
  for (int j = 0; j < 2; j++) {
    const double s_term = sphi_n[j] * p.sphi;
    const double c_term = cphi_n[j] * p.cphi;
    double cospsi[2];
#pragma unroll
    for (int i = 0; i < 2; i++) cospsi[i] = fma(c_term, coslambda[i], s_term);
#pragma unroll
    for (int k = 0; k < 2; k++) {
      const double dr = p.r - r_n[k];
      const double dr2 = dr * dr;
      const double rr = two_r * r_n[k];
#pragma unroll
      for (int i = 0; i < 2; i++) {
        const double inv = lean::lm_rsqrt(fma(rr, 1.0 - cospsi[i], dr2));
        const double m = mass[(j * 2 + k) * 2 + i];
        if (FIELD == 0) {
          result = fma(m, inv, result);
        } else {
          const double delta_z = fma(-r_n[k], cospsi[i], p.r);
          result = fma(m * delta_z, (inv * inv) * inv, result);
        }
      }
    }
  }
  // G (and the sign of gravity_u_spherical) applied once per tesseroid
  return FIELD == 0 ? result * kG : result * -kG;
}

// _adaptive_discretization (_tesseroid_utils.py:150-241) for one pair, each
// small tesseroid integrated when popped (the order in which the reference
// stores and then integrates them).  status: 1 stack overflow, 2 more than
// MAX_DISCRETIZATIONS small tesseroids.
template <int FIELD>
__device__ __noinline__ double adaptive_pair(const Station& p, const double* root, double density,
                                             const Adapt& ad, const GlqRule& q, int& status) {
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
      acc = add(acc, glq_eval<FIELD>(p, nd.lon, nd.cphi, nd.sphi, nd.r, nd.mass));
    }
  }
  return acc;
}

__global__ void prepare_kernel(const double* __restrict__ aos, const double* __restrict__ density,
                               int64_t m, double* __restrict__ rec, int64_t stride, double ratio,
                               GlqRule q) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= m) return;
  double t[6];
#pragma unroll
  for (int c = 0; c < 6; c++) t[c] = aos[6 * j + c];
  const double rho = density[j];
#pragma unroll
  for (int c = 0; c < 6; c++) rec[c * stride + j] = t[c];
  rec[kRho * stride + j] = rho;
  // _discard_null_tesseroids (_tesseroid_utils.py:503-538)
  const bool null = t[0] == t[1] || t[2] == t[3] || t[4] == t[5] || rho == 0.0;
  rec[kSkip * stride + j] = null ? 1.0 : 0.0;
  double l[3];
  dimensions(t, l[0], l[1], l[2]);
#pragma unroll
  for (int a = 0; a < 3; a++) {
    rec[(kLLon + a) * stride + j] = l[a];
    const double far = mul(mul(ratio, l[a]), kPreTest);
    rec[(kFar2Lon + a) * stride + j] = l[a] > 0.0 ? far * far : INFINITY;
  }
  double lon_c, cos_c, sin_c, r_c;
  centre(t, lon_c, cos_c, sin_c, r_c);
  rec[kLonC * stride + j] = lon_c;
  rec[kCosC * stride + j] = cos_c;
  rec[kSinC * stride + j] = sin_c;
  rec[kRC * stride + j] = r_c;
  double s_lon_c, c_lon_c;
  sincos(lon_c, &s_lon_c, &c_lon_c);
  rec[kCosLonC * stride + j] = c_lon_c;
  rec[kSinLonC * stride + j] = s_lon_c;
  Nodes nd;
  glq_nodes(t, rho, q, nd);
#pragma unroll
  for (int a = 0; a < 2; a++) {
    double s_lon, c_lon;
    sincos(nd.lon[a], &s_lon, &c_lon);
    rec[(kNodeCosLon + a) * stride + j] = c_lon;
    rec[(kNodeSinLon + a) * stride + j] = s_lon;
    rec[(kNodeCos + a) * stride + j] = nd.cphi[a];
    rec[(kNodeSin + a) * stride + j] = nd.sphi[a];
    rec[(kNodeRad + a) * stride + j] = nd.r[a];
  }
#pragma unroll
  for (int a = 0; a < 8; a++) rec[(kMass + a) * stride + j] = nd.mass[a];
}

// Run the queued split pairs of this warp, 32 at a time (one per lane), and
// add each result to its point's sum in list order.
template <int FIELD>
__device__ __forceinline__ void flush_near(const uint32_t* list, int count, int lane,
                                           const Station& mine, const double* __restrict__ rec,
                                           int64_t stride, int64_t p0, const Adapt& ad,
                                           const GlqRule& q, double& acc, int& status) {
  for (int r0 = 0; r0 < count; r0 += 32) {
    const int e = r0 + lane;
    const bool has = e < count;
    const uint32_t ent = has ? list[e] : 0u;
    const int owner = has ? (int)(ent & 31u) : lane;
    Station s;
    s.lon = __shfl_sync(0xffffffffu, mine.lon, owner);
    s.cphi = __shfl_sync(0xffffffffu, mine.cphi, owner);
    s.sphi = __shfl_sync(0xffffffffu, mine.sphi, owner);
    s.r = __shfl_sync(0xffffffffu, mine.r, owner);
    s.clon = __shfl_sync(0xffffffffu, mine.clon, owner);
    s.slon = __shfl_sync(0xffffffffu, mine.slon, owner);
    double contrib = 0.0;
    if (has) {
      const int64_t j = p0 + (int64_t)(ent >> 5);
      double root[6];
#pragma unroll
      for (int c = 0; c < 6; c++) root[c] = rec[c * stride + j];
      contrib = adaptive_pair<FIELD>(s, root, rec[kRho * stride + j], ad, q, status);
    }
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

template <int FIELD>
__global__ void __launch_bounds__(kThreads) forward_kernel(
    const double* __restrict__ lon_deg, const double* __restrict__ lat_deg,
    const double* __restrict__ radius, int64_t n_obs, const double* __restrict__ rec,
    int64_t stride, int64_t n_tess, int64_t chunk, Adapt ad, GlqRule q,
    double* __restrict__ dst, int64_t dst_chunk_stride, double out_scale,
    int32_t* __restrict__ status_out) {
  __shared__ double sh[kSmemRows][kTile];
  __shared__ uint32_t near_list[kWarps][kNearCap];
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int64_t i = (int64_t)blockIdx.x * kThreads + threadIdx.x;
  const bool active = i < n_obs;
  Station p;
  p.lon = rad(active ? lon_deg[i] : 0.0);
  sincos(rad(active ? lat_deg[i] : 0.0), &p.sphi, &p.cphi);
  sincos(p.lon, &p.slon, &p.clon);
  p.r = active ? radius[i] : 1.0;
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
      if (sh[kSkip - kLonC][c] != 0.0) continue;  // same for the whole block
      bool near = false;
      if (active) {
#define S(row) sh[(row) - kLonC][c]
        // squared distance to the centre from the longitude cosines/sines; it
        // differs from the reference's by at most `slack`, so d2 - slack >=
        // far^2 proves distance / size >= ratio on that axis
        const double r_c = S(kRC);
        const double clam = fma(S(kCosLonC), p.clon, S(kSinLonC) * p.slon);
        const double cospsi_c = fma(S(kCosC) * p.cphi, clam, S(kSinC) * p.sphi);
        const double dr_c = p.r - r_c;
        const double rr_c = 2.0 * p.r * r_c;
        const double d2 = fma(rr_c, 1.0 - cospsi_c, dr_c * dr_c);
        const double lo = d2 - fma(fabs(rr_c), 4e-15, d2 * 4e-15);
        if (!(lo >= S(kFar2Lon)) || !(lo >= S(kFar2Lat)) || (rad_split && !(lo >= S(kFar2Rad)))) {
          // undecided: the reference's distance and quotients
          double cospsi;
          const double d = distance_core(p, S(kLonC), S(kCosC), S(kSinC), r_c, cospsi);
          near = split_axis(d, S(kLLon), ratio) || split_axis(d, S(kLLat), ratio) ||
                 (rad_split && split_axis(d, S(kLRad), ratio));
        }
        if (!near) {
          const double clon_n[2] = {S(kNodeCosLon), S(kNodeCosLon + 1)};
          const double slon_n[2] = {S(kNodeSinLon), S(kNodeSinLon + 1)};
          const double cphi_n[2] = {S(kNodeCos), S(kNodeCos + 1)};
          const double sphi_n[2] = {S(kNodeSin), S(kNodeSin + 1)};
          const double r_n[2] = {S(kNodeRad), S(kNodeRad + 1)};
          double mass[8];
#pragma unroll
          for (int a = 0; a < 8; a++) mass[a] = S(kMass + a);
          acc += glq_eval_fast<FIELD>(p, clon_n, slon_n, cphi_n, sphi_n, r_n, mass);
        }
#undef S
      }
      const unsigned ball = __ballot_sync(0xffffffffu, near);
      if (ball) {
        const int add_n = __popc(ball);
        if (n_near + add_n > kNearCap) {
          flush_near<FIELD>(near_list[warp], n_near, lane, p, rec, stride, p0, ad, q, acc,
                            status);
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
  if (n_near > 0)
    flush_near<FIELD>(near_list[warp], n_near, lane, p, rec, stride, p0, ad, q, acc, status);
  if (status && status_out) atomicOr(status_out, status);
  if (active) dst[(int64_t)blockIdx.y * dst_chunk_stride + i] = mul(acc, out_scale);
}

__global__ void reduce_kernel(const double* __restrict__ part, int64_t n_chunks, int64_t n_obs,
                              double scale, double* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_obs) return;
  double s = 0.0;
  for (int64_t c = 0; c < n_chunks; c++) s = add(s, part[c * n_obs + i]);
  out[i] = mul(s, scale);
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
    if (!active) continue;
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
  size_t rec_bytes, part_bytes;
};

Plan make_plan(int64_t n_obs, int64_t m) {
  Plan p;
  p.n_tiles = (n_obs + kThreads - 1) / kThreads;
  if (p.n_tiles < 1) p.n_tiles = 1;
  int64_t m_tiles = (m + kTile - 1) / kTile;
  if (m_tiles < 1) m_tiles = 1;
  const int64_t target = (int64_t)kSms * 8;
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
  *bytes = p.rec_bytes + p.part_bytes;
  return HG_OK;
}

int hg_tesseroid_forward(const double* longitude, const double* latitude, const double* radius,
                         int64_t n_obs, const double* tesseroids, const double* density,
                         int64_t n_tesseroids, int32_t field, int32_t radial_discretization,
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
  const size_t need = plan.rec_bytes + plan.part_bytes;
  bool own = false;
  if (workspace == nullptr) {
    cudaError_t e = cudaMallocAsync(&workspace, need, st);
    if (e != cudaSuccess) return cuda_check(e, "cudaMallocAsync(workspace)");
    own = true;
  } else if (workspace_bytes < need) {
    return set_error(HG_ERR_INVALID, "workspace too small");
  }
  double* rec = static_cast<double*>(workspace);
  double* part = reinterpret_cast<double*>(static_cast<char*>(workspace) + plan.rec_bytes);
  const tess::GlqRule q = tess::make_rule(glq_nodes, glq_weights);
  tess::Adapt ad;
  ad.ratio = field == 3 ? 2.5 : 1.0;  // DISTANCE_SIZE_RATII, tesseroid_gravity.py:30
  ad.radial = radial_discretization ? 1 : 0;
  ad.stack_size = stack_size > 0 ? stack_size : tess::kStackSize;
  ad.max_leaves = max_discretizations > 0 ? max_discretizations : tess::kMaxLeaves;
  const int threads = 256;
  tess::prepare_kernel<<<(unsigned)((n_tesseroids + threads - 1) / threads), threads, 0, st>>>(
      tesseroids, density, n_tesseroids, rec, n_tesseroids, ad.ratio, q);
  int rc = cuda_check(cudaGetLastError(), "tesseroid prepare_kernel launch");
  if (rc == HG_OK) {
    const bool direct = plan.n_chunks == 1;
    double* dst = direct ? out : part;
    const dim3 grid((unsigned)plan.n_tiles, (unsigned)plan.n_chunks);
    if (field == 0)
      tess::forward_kernel<0><<<grid, tess::kThreads, 0, st>>>(
          longitude, latitude, radius, n_obs, rec, n_tesseroids, n_tesseroids, plan.chunk, ad, q,
          dst, n_obs, direct ? scale : 1.0, status);
    else
      tess::forward_kernel<1><<<grid, tess::kThreads, 0, st>>>(
          longitude, latitude, radius, n_obs, rec, n_tesseroids, n_tesseroids, plan.chunk, ad, q,
          dst, n_obs, direct ? scale : 1.0, status);
    rc = cuda_check(cudaGetLastError(), "tesseroid forward_kernel launch");
    if (rc == HG_OK && !direct) {
      tess::reduce_kernel<<<(unsigned)((n_obs + threads - 1) / threads), threads, 0, st>>>(
          part, plan.n_chunks, n_obs, scale, out);
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
