// Point-mass gravity: all-pairs sum over observation points x point masses
// (harmonica src/harmonica/_forward/point.py, point_mass_cartesian :357-398
// and point_mass_spherical :400-450).  Same work decomposition as the prism
// kernels: one thread per observation point, point masses staged in shared
// memory, prism-chunk partials replaced by point-chunk partials reduced in
// fixed order.  FP64, with the FP32-seeded reciprocal square root.
//
// Cartesian kernels (choclo.point, from V = G m / l): with d = P - Q,
//   potential  G m / l;   g_a = -G m d_a / l^3;
//   g_ab = G m (3 d_a d_b - delta_ab l^2) / l^5.
// The kernel returns them divided by G m and, for the first derivatives, by
// -G m, the convention of field_scale() shared with the prism kernels.
// Spherical (longitude, latitude in degrees, radius): potential G m / l and
// the upward component -G m (r - r_p cos psi) / l^3 with
//   cos psi = sin phi_p sin phi + cos phi_p cos phi cos(lambda_p - lambda),
//   l = sqrt((r - r_p)^2 + 2 r r_p (1 - cos psi))      (utils.py:164-201).
#include <cuda_runtime.h>

#include <string>

#include "../../include/harmonica_gb300.h"
#include "forward_core.cuh"
#include "lean_packed.cuh"

namespace hg {

int set_error(int code, const std::string& msg);
int cuda_check(cudaError_t e, const char* what);

namespace {

struct PointTile {
  double a[kTile], b[kTile], c[kTile], d[kTile], m[kTile];
};

constexpr double kDeg = 3.141592653589793 / 180.0;

template <int F>
__device__ __forceinline__ double point_cart(double dx, double dy, double dz) {
  const double l2 = fma(dx, dx, fma(dy, dy, dz * dz));
  const double inv = lean::lm_rsqrt(l2);
  if (F == kPotential) return inv;
  const double inv3 = (inv * inv) * inv;
  // first derivatives carry the sign convention of the prism combinations
  // (field_scale applies -G for them): +d / l^3 here is -g_a / (G m)
  if (F == kGe) return dx * inv3;
  if (F == kGn) return dy * inv3;
  if (F == kGz) return dz * inv3;
  const double inv5 = inv3 * (inv * inv);
  if (F == kGee) return fma(3.0 * dx, dx, -l2) * inv5;
  if (F == kGnn) return fma(3.0 * dy, dy, -l2) * inv5;
  if (F == kGzz) return fma(3.0 * dz, dz, -l2) * inv5;
  if (F == kGen) return 3.0 * dx * dy * inv5;
  if (F == kGez) return 3.0 * dx * dz * inv5;
  return 3.0 * dy * dz * inv5;  // kGnz
}

// SPH: 0 Cartesian (coordinates e, n, u), 1 spherical (lon, lat, r in degrees/m)
template <int F, int SPH>
__global__ void __launch_bounds__(kThreads) point_kernel(
    const double* __restrict__ c1, const double* __restrict__ c2, const double* __restrict__ c3,
    int64_t n_obs, const double* __restrict__ p1, const double* __restrict__ p2,
    const double* __restrict__ p3, const double* __restrict__ mass, int64_t n_points,
    int64_t chunk, double* __restrict__ dst, int64_t dst_chunk_stride, double out_scale) {
  __shared__ PointTile sh;
  const int64_t i = (int64_t)blockIdx.x * kThreads + threadIdx.x;
  const bool active = i < n_obs;
  double x1 = active ? c1[i] : 0.0, x2 = active ? c2[i] : 0.0, x3 = active ? c3[i] : 1.0;
  double cphi = 0.0, sphi = 0.0;
  if (SPH) {
    x1 *= kDeg;
    sincos(x2 * kDeg, &sphi, &cphi);
  }
  double acc = 0.0;
  const int64_t q0 = (int64_t)blockIdx.y * chunk;
  const int64_t q1 = min(q0 + chunk, n_points);
  for (int64_t base = q0; base < q1; base += kTile) {
    const int cnt = (int)min((int64_t)kTile, q1 - base);
    __syncthreads();
    if ((int)threadIdx.x < cnt) {
      const int64_t j = base + threadIdx.x;
      if (SPH) {
        double sp, cp;
        sincos(p2[j] * kDeg, &sp, &cp);
        sh.a[threadIdx.x] = p1[j] * kDeg;
        sh.b[threadIdx.x] = cp;
        sh.c[threadIdx.x] = sp;
        sh.d[threadIdx.x] = p3[j];
      } else {
        sh.a[threadIdx.x] = p1[j];
        sh.b[threadIdx.x] = p2[j];
        sh.c[threadIdx.x] = p3[j];
      }
      sh.m[threadIdx.x] = mass[j];
    }
    __syncthreads();
    for (int k = 0; k < cnt; k++) {
      double v;
      if (SPH) {
        const double coslambda = cos(sh.a[k] - x1);
        const double cospsi = sh.c[k] * sphi + sh.b[k] * cphi * coslambda;
        const double rp = sh.d[k];
        const double dr = x3 - rp;
        const double l2 = dr * dr + 2.0 * x3 * rp * (1.0 - cospsi);
        const double inv = lean::lm_rsqrt(l2);
        v = F == kPotential ? inv : (x3 - rp * cospsi) * ((inv * inv) * inv);
      } else {
        v = point_cart<F>(x1 - sh.a[k], x2 - sh.b[k], x3 - sh.c[k]);
      }
      acc = fma(sh.m[k], v, acc);
    }
  }
  if (!active) return;
  dst[(int64_t)blockIdx.y * dst_chunk_stride + i] = acc * out_scale;
}

// Cartesian potential and first derivatives on packed float pairs (the
// point-mass analogue of the tesseroid kernel's fast path): the coordinates
// of points and masses, taken relative to the first point in FP64, become
// 48-bit float pairs; per pair of masses (the two lanes of a float2) the
// difference d = P - Q, l^2 = |d|^2, 1 / l by a float-pair reciprocal square
// root and m / l or m d_a / l^3 (the quantities of point_cart) on
// FFMA2/FADD2/FMUL2, summed on float pairs over a tile and added to the FP64
// accumulator per tile.  Each term's relative error is the 48-bit rounding
// of the coordinates, ~2^-48 x (distance of the points from the first point)
// / d, plus a few 2^-46: 4e-11 for d = 10 m at 1e5 m from the first point,
// 1e-13 at 10 km (tests/test_float_pairs.py; the parity tests' tolerance is
// 1e-10); the FP64 pipe, 1/64 of the FP32 rate here, only sees the per-tile
// sums.
struct PointTileF2 {
  float xh[kTile], xl[kTile], yh[kTile], yl[kTile], zh[kTile], zl[kTile], mh[kTile], ml[kTile];
};

template <int F>
__global__ void __launch_bounds__(kThreads) point_pairs_kernel(
    const double* __restrict__ c1, const double* __restrict__ c2, const double* __restrict__ c3,
    int64_t n_obs, const double* __restrict__ p1, const double* __restrict__ p2,
    const double* __restrict__ p3, const double* __restrict__ mass, int64_t n_points,
    int64_t chunk, double* __restrict__ dst, int64_t dst_chunk_stride, double out_scale) {
  using namespace lean;
  __shared__ PointTileF2 sh;
  const int64_t i = (int64_t)blockIdx.x * kThreads + threadIdx.x;
  const bool active = i < n_obs;
  const double o1 = c1[0], o2 = c2[0], o3 = c3[0];  // origin: the first point
  const F2 px = double_to_f2(active ? c1[i] - o1 : 0.0);
  const F2 py = double_to_f2(active ? c2[i] - o2 : 0.0);
  const F2 pz = double_to_f2(active ? c3[i] - o3 : 0.0);
  const P2 X{sp2(px.h), sp2(px.l)}, Y{sp2(py.h), sp2(py.l)}, Z{sp2(pz.h), sp2(pz.l)};
  double acc = 0.0;
  const int64_t q0 = (int64_t)blockIdx.y * chunk;
  const int64_t q1 = min(q0 + chunk, n_points);
  for (int64_t base = q0; base < q1; base += kTile) {
    const int cnt = (int)min((int64_t)kTile, q1 - base);
    __syncthreads();
    {
      const int t = threadIdx.x;
      F2 qx{1e15f, 0.0f}, qy{0.0f, 0.0f}, qz{0.0f, 0.0f}, qm{0.0f, 0.0f};  // padding: far, massless
      if (t < cnt) {
        const int64_t j = base + t;
        qx = double_to_f2(p1[j] - o1);
        qy = double_to_f2(p2[j] - o2);
        qz = double_to_f2(p3[j] - o3);
        qm = double_to_f2(mass[j]);
      }
      sh.xh[t] = qx.h; sh.xl[t] = qx.l; sh.yh[t] = qy.h; sh.yl[t] = qy.l;
      sh.zh[t] = qz.h; sh.zl[t] = qz.l; sh.mh[t] = qm.h; sh.ml[t] = qm.l;
    }
    __syncthreads();
    const auto lane2 = [](const float* a, int k) {
      return *reinterpret_cast<const float2*>(&a[2 * k]);
    };
    P2 sum{sp2(0.0f), sp2(0.0f)};
    const int npair = (cnt + 1) / 2;
    for (int k = 0; k < npair; k++) {
      const P2 dx = p2_diff(X, P2{lane2(sh.xh, k), lane2(sh.xl, k)});
      const P2 dy = p2_diff(Y, P2{lane2(sh.yh, k), lane2(sh.yl, k)});
      const P2 dz = p2_diff(Z, P2{lane2(sh.zh, k), lane2(sh.zl, k)});
      const P2 inv = p2_rsqrt(p2_norm2(dx, dy, dz));
      const P2 m{lane2(sh.mh, k), lane2(sh.ml, k)};
      P2 term;
      if (F == kPotential) {
        term = p2_mul(m, inv);
      } else {
        const P2 da = F == kGe ? dx : (F == kGn ? dy : dz);
        term = p2_mul(p2_mul(m, da), p2_mul(p2_mul(inv, inv), inv));
      }
      const P2 s2 = two_sum2(sum.h, term.h);
      sum = P2{s2.h, add2(sum.l, add2(s2.l, term.l))};
    }
    acc += f2_to_double(f2_add(F2{sum.h.x, sum.l.x}, F2{sum.h.y, sum.l.y}), 0);
  }
  if (!active) return;
  dst[(int64_t)blockIdx.y * dst_chunk_stride + i] = acc * out_scale;
}

// Magnetic field of dipoles (src/harmonica/_forward/dipole.py:23-130,
// 292-360, with choclo.dipole's closed form): with r = P - Q,
// b = mu0/(4 pi) (3 (m . r) r / l^5 - m / l^3); the kernel sums
// (3 (m . r) r_a - m_a l^2) / l^5 and the reduction applies mu0/(4 pi) and
// nT.  COMP 0/1/2: b_e, b_n, b_u; 3: all three (rows e, n, u).
struct DipoleTile {
  double e[kTile], n[kTile], u[kTile], me[kTile], mn[kTile], mu[kTile];
};

template <int COMP>
__global__ void __launch_bounds__(kThreads) dipole_kernel(
    const double* __restrict__ oe, const double* __restrict__ on, const double* __restrict__ ou,
    int64_t n_obs, const double* __restrict__ de, const double* __restrict__ dn,
    const double* __restrict__ du, const double* __restrict__ me, const double* __restrict__ mn,
    const double* __restrict__ mu, int64_t n_dip, int64_t chunk, double* __restrict__ dst,
    int64_t dst_chunk_stride, double out_scale) {
  __shared__ DipoleTile sh;
  const int64_t i = (int64_t)blockIdx.x * kThreads + threadIdx.x;
  const bool active = i < n_obs;
  const double pe = active ? oe[i] : 0.0, pn = active ? on[i] : 0.0, pu = active ? ou[i] : 0.0;
  double be = 0.0, bn = 0.0, bu = 0.0;
  const int64_t q0 = (int64_t)blockIdx.y * chunk;
  const int64_t q1 = min(q0 + chunk, n_dip);
  for (int64_t base = q0; base < q1; base += kTile) {
    const int cnt = (int)min((int64_t)kTile, q1 - base);
    __syncthreads();
    if ((int)threadIdx.x < cnt) {
      const int64_t j = base + threadIdx.x;
      sh.e[threadIdx.x] = de[j];
      sh.n[threadIdx.x] = dn[j];
      sh.u[threadIdx.x] = du[j];
      sh.me[threadIdx.x] = me[j];
      sh.mn[threadIdx.x] = mn[j];
      sh.mu[threadIdx.x] = mu[j];
    }
    __syncthreads();
    for (int k = 0; k < cnt; k++) {
      const double rx = pe - sh.e[k], ry = pn - sh.n[k], rz = pu - sh.u[k];
      const double l2 = fma(rx, rx, fma(ry, ry, rz * rz));
      const double inv = lean::lm_rsqrt(l2);
      const double inv2 = inv * inv;
      const double inv5 = (inv2 * inv2) * inv;
      const double mdr3 = 3.0 * fma(sh.me[k], rx, fma(sh.mn[k], ry, sh.mu[k] * rz));
      if (COMP == 0 || COMP == 3) be = fma(fma(mdr3, rx, -sh.me[k] * l2), inv5, be);
      if (COMP == 1 || COMP == 3) bn = fma(fma(mdr3, ry, -sh.mn[k] * l2), inv5, bn);
      if (COMP == 2 || COMP == 3) bu = fma(fma(mdr3, rz, -sh.mu[k] * l2), inv5, bu);
    }
  }
  if (!active) return;
  double* d = dst + (int64_t)blockIdx.y * dst_chunk_stride;
  if (COMP == 3) {
    d[i] = be * out_scale;
    d[n_obs + i] = bn * out_scale;
    d[2 * n_obs + i] = bu * out_scale;
  } else {
    d[i] = (COMP == 0 ? be : (COMP == 1 ? bn : bu)) * out_scale;
  }
}

// One row block of the equivalent-source Jacobian: jac[i][j] = 1 / l(i, j),
// greens_func_cartesian / greens_func_spherical (src/harmonica/
// _equivalent_sources/cartesian.py:635-644, spherical.py:413-424) filled by
// the loop of jacobian (_equivalent_sources/utils.py:54-74).  Threads run
// along the sources, so each row is written in coalesced 256-byte pieces;
// a block covers kJacRows points.
constexpr int kJacRows = 8;

template <int SPH>
__global__ void __launch_bounds__(kThreads) jacobian_kernel(
    const double* __restrict__ c1, const double* __restrict__ c2, const double* __restrict__ c3,
    int64_t n_obs, const double* __restrict__ p1, const double* __restrict__ p2,
    const double* __restrict__ p3, int64_t n_points, double* __restrict__ jac) {
  const int64_t j = (int64_t)blockIdx.x * kThreads + threadIdx.x;
  if (j >= n_points) return;
  double a = p1[j], b = p2[j], c = p3[j];
  if (SPH) {
    double sp, cp;
    sincos(b * kDeg, &sp, &cp);
    a *= kDeg;
    b = cp;
    c = sp;
  }
  const double rp = SPH ? p3[j] : 0.0;
  const int64_t i0 = (int64_t)blockIdx.y * kJacRows;
  const int64_t i1 = min(i0 + kJacRows, n_obs);
  for (int64_t i = i0; i < i1; i++) {
    double l2;
    if (SPH) {
      double sphi, cphi;
      sincos(c2[i] * kDeg, &sphi, &cphi);
      const double r = c3[i];
      const double cospsi = c * sphi + b * cphi * cos(a - c1[i] * kDeg);
      const double dr = r - rp;
      l2 = dr * dr + 2.0 * r * rp * (1.0 - cospsi);
    } else {
      const double dx = c1[i] - a, dy = c2[i] - b, dz = c3[i] - c;
      l2 = fma(dx, dx, fma(dy, dy, dz * dz));
    }
    jac[i * n_points + j] = lean::lm_rsqrt(l2);
  }
}

struct PointPlan {
  int64_t tiles, n_chunks, chunk;
  size_t bytes;
};

PointPlan point_plan(int64_t n_obs, int64_t n_points) {
  PointPlan p;
  p.tiles = (n_obs + kThreads - 1) / kThreads;
  const int64_t target = (int64_t)kSmCount * 4 * launch_waves();
  int64_t pt = (n_points + kTile - 1) / kTile;
  if (pt < 1) pt = 1;
  int64_t want = (target + (p.tiles > 0 ? p.tiles : 1) - 1) / (p.tiles > 0 ? p.tiles : 1);
  want = want < 1 ? 1 : (want > pt ? pt : want);
  if (want > 65535) want = 65535;
  p.chunk = ((pt + want - 1) / want) * kTile;
  p.n_chunks = n_points > 0 ? (n_points + p.chunk - 1) / p.chunk : 1;
  p.bytes = p.n_chunks > 1 ? (size_t)p.n_chunks * (size_t)n_obs * sizeof(double) : 0;
  return p;
}

// unit: the sum of m / l without G (the equivalent-source prediction,
// _equivalent_sources/utils.py:77-96); only for the potential kernel.
template <int SPH>
int launch_point(int field, const double* c1, const double* c2, const double* c3, int64_t n_obs,
                 const double* p1, const double* p2, const double* p3, const double* m,
                 int64_t n_points, double* out, void* ws, size_t ws_bytes, cudaStream_t st,
                 bool unit = false) {
  const PointPlan plan = point_plan(n_obs, n_points);
  if (n_obs == 0) return HG_OK;
  if (n_points == 0)
    return cuda_check(cudaMemsetAsync(out, 0, sizeof(double) * n_obs, st), "cudaMemsetAsync");
  const bool direct = plan.n_chunks == 1;
  if (!direct && (!ws || ws_bytes < plan.bytes))
    return set_error(HG_ERR_INVALID, "workspace missing or too small");
  double* dst = direct ? out : static_cast<double*>(ws);
  const double scale = unit ? 1.0 : field_scale(field);
  dim3 grid((unsigned)plan.tiles, (unsigned)plan.n_chunks);
  switch (field) {
#define HG_PT(FF)                                                                              \
  case FF:                                                                                     \
    if (!SPH && FF <= kGz)                                                                     \
      point_pairs_kernel<FF><<<grid, kThreads, 0, st>>>(c1, c2, c3, n_obs, p1, p2, p3, m,      \
                                                        n_points, plan.chunk, dst, n_obs,      \
                                                        direct ? scale : 1.0);                 \
    else                                                                                       \
      point_kernel<FF, SPH><<<grid, kThreads, 0, st>>>(c1, c2, c3, n_obs, p1, p2, p3, m,      \
                                                        n_points, plan.chunk, dst, n_obs,      \
                                                        direct ? scale : 1.0);                 \
    break;
    HG_PT(0) HG_PT(1) HG_PT(2) HG_PT(3) HG_PT(4) HG_PT(5) HG_PT(6) HG_PT(7) HG_PT(8) HG_PT(9)
#undef HG_PT
    default: return set_error(HG_ERR_INVALID, "bad field");
  }
  int rc = cuda_check(cudaGetLastError(), "point_kernel launch");
  if (rc != HG_OK || direct) return rc;
  launch_chunk_sum(dst, plan.n_chunks, n_obs, n_obs, scale, out, st);
  return cuda_check(cudaGetLastError(), "chunk_sum_kernel launch");
}

}  // namespace
}  // namespace hg

using namespace hg;

extern "C" {

int hg_point_forward_workspace(int64_t n_obs, int64_t n_points, size_t* bytes) {
  if (!bytes || n_obs < 0 || n_points < 0) return set_error(HG_ERR_INVALID, "bad arguments");
  *bytes = point_plan(n_obs, n_points).bytes;
  return HG_OK;
}

int hg_point_forward(const double* obs_1, const double* obs_2, const double* obs_3,
                     int64_t n_obs, const double* pts_1, const double* pts_2,
                     const double* pts_3, const double* masses, int64_t n_points,
                     int32_t spherical, int32_t field, double* out, void* workspace,
                     size_t workspace_bytes, void* stream) {
  if (n_obs < 0 || n_points < 0 || field < 0 || field >= kNumFields)
    return set_error(HG_ERR_INVALID, "bad sizes or field");
  if (spherical && field != kPotential && field != kGz)
    return set_error(HG_ERR_INVALID, "spherical point masses: potential and g_z only");
  if (n_obs > 0 && (!obs_1 || !obs_2 || !obs_3 || !out))
    return set_error(HG_ERR_INVALID, "null pointer");
  if (n_points > 0 && (!pts_1 || !pts_2 || !pts_3 || !masses))
    return set_error(HG_ERR_INVALID, "null points pointer");
  cudaStream_t st = (cudaStream_t)stream;
  if (spherical)
    return launch_point<1>(field, obs_1, obs_2, obs_3, n_obs, pts_1, pts_2, pts_3, masses,
                           n_points, out, workspace, workspace_bytes, st);
  return launch_point<0>(field, obs_1, obs_2, obs_3, n_obs, pts_1, pts_2, pts_3, masses,
                         n_points, out, workspace, workspace_bytes, st);
}

int hg_dipole_workspace(int64_t n_obs, int64_t n_dipoles, int32_t component, size_t* bytes) {
  if (!bytes || n_obs < 0 || n_dipoles < 0 || component < 0 || component > 3)
    return set_error(HG_ERR_INVALID, "bad arguments");
  const PointPlan p = point_plan(n_obs, n_dipoles);
  *bytes = p.n_chunks > 1 ? p.bytes * (component == 3 ? 3 : 1) : 0;
  return HG_OK;
}

int hg_dipole_magnetic(const double* obs_e, const double* obs_n, const double* obs_u,
                       int64_t n_obs, const double* dip_e, const double* dip_n,
                       const double* dip_u, const double* m_e, const double* m_n,
                       const double* m_u, int64_t n_dipoles, int32_t component, double* out,
                       void* workspace, size_t workspace_bytes, void* stream) {
  if (n_obs < 0 || n_dipoles < 0 || component < 0 || component > 3)
    return set_error(HG_ERR_INVALID, "bad sizes or component");
  if (n_obs == 0) return HG_OK;
  if (!obs_e || !obs_n || !obs_u || !out) return set_error(HG_ERR_INVALID, "null pointer");
  if (n_dipoles > 0 && (!dip_e || !dip_n || !dip_u || !m_e || !m_n || !m_u))
    return set_error(HG_ERR_INVALID, "null dipole pointer");
  cudaStream_t st = (cudaStream_t)stream;
  const int rows = component == 3 ? 3 : 1;
  if (n_dipoles == 0)
    return cuda_check(cudaMemsetAsync(out, 0, sizeof(double) * rows * n_obs, st),
                      "cudaMemsetAsync");
  const PointPlan plan = point_plan(n_obs, n_dipoles);
  const bool direct = plan.n_chunks == 1;
  const size_t need = direct ? 0 : plan.bytes * rows;
  if (!direct && (!workspace || workspace_bytes < need))
    return set_error(HG_ERR_INVALID, "workspace missing or too small");
  // mu0 / (4 pi) = 1e-7 H/m, results in nT (dipole.py:193-195)
  const double scale = 1e-7 * 1e9;
  double* dst = direct ? out : static_cast<double*>(workspace);
  const int64_t cstride = (int64_t)rows * n_obs;
  const dim3 grid((unsigned)plan.tiles, (unsigned)plan.n_chunks);
  const double sc = direct ? scale : 1.0;
  switch (component) {
    case 0: dipole_kernel<0><<<grid, kThreads, 0, st>>>(obs_e, obs_n, obs_u, n_obs, dip_e, dip_n, dip_u, m_e, m_n, m_u, n_dipoles, plan.chunk, dst, cstride, sc); break;
    case 1: dipole_kernel<1><<<grid, kThreads, 0, st>>>(obs_e, obs_n, obs_u, n_obs, dip_e, dip_n, dip_u, m_e, m_n, m_u, n_dipoles, plan.chunk, dst, cstride, sc); break;
    case 2: dipole_kernel<2><<<grid, kThreads, 0, st>>>(obs_e, obs_n, obs_u, n_obs, dip_e, dip_n, dip_u, m_e, m_n, m_u, n_dipoles, plan.chunk, dst, cstride, sc); break;
    default: dipole_kernel<3><<<grid, kThreads, 0, st>>>(obs_e, obs_n, obs_u, n_obs, dip_e, dip_n, dip_u, m_e, m_n, m_u, n_dipoles, plan.chunk, dst, cstride, sc); break;
  }
  int rc = cuda_check(cudaGetLastError(), "dipole_kernel launch");
  if (rc != HG_OK || direct) return rc;
  launch_chunk_sum(dst, plan.n_chunks, cstride, cstride, scale, out, st);
  return cuda_check(cudaGetLastError(), "chunk_sum_kernel launch");
}

int hg_eqs_jacobian(const double* obs_1, const double* obs_2, const double* obs_3, int64_t n_obs,
                    const double* pts_1, const double* pts_2, const double* pts_3,
                    int64_t n_points, int32_t spherical, double* jac, void* stream) {
  if (n_obs < 0 || n_points < 0) return set_error(HG_ERR_INVALID, "bad sizes");
  if (n_obs == 0 || n_points == 0) return HG_OK;
  if (!obs_1 || !obs_2 || !obs_3 || !pts_1 || !pts_2 || !pts_3 || !jac)
    return set_error(HG_ERR_INVALID, "null pointer");
  const int64_t col_blocks = (n_points + kThreads - 1) / kThreads;
  const int64_t row_blocks = (n_obs + kJacRows - 1) / kJacRows;
  if (col_blocks > 2147483647LL || row_blocks > 65535LL * 65535LL)
    return set_error(HG_ERR_INVALID, "Jacobian too large for one launch");
  cudaStream_t st = (cudaStream_t)stream;
  // rows in launches of at most 65535 row blocks (the grid's y limit)
  for (int64_t r0 = 0; r0 < row_blocks; r0 += 65535) {
    const int64_t nb = min(row_blocks - r0, (int64_t)65535);
    const int64_t first = r0 * kJacRows;
    const dim3 grid((unsigned)col_blocks, (unsigned)nb);
    if (spherical)
      jacobian_kernel<1><<<grid, kThreads, 0, st>>>(obs_1 + first, obs_2 + first, obs_3 + first,
                                                    n_obs - first, pts_1, pts_2, pts_3, n_points,
                                                    jac + first * n_points);
    else
      jacobian_kernel<0><<<grid, kThreads, 0, st>>>(obs_1 + first, obs_2 + first, obs_3 + first,
                                                    n_obs - first, pts_1, pts_2, pts_3, n_points,
                                                    jac + first * n_points);
    const int rc = cuda_check(cudaGetLastError(), "jacobian_kernel launch");
    if (rc != HG_OK) return rc;
  }
  return HG_OK;
}

int hg_eqs_predict(const double* obs_1, const double* obs_2, const double* obs_3, int64_t n_obs,
                   const double* pts_1, const double* pts_2, const double* pts_3,
                   const double* coefs, int64_t n_points, int32_t spherical, double* out,
                   void* workspace, size_t workspace_bytes, void* stream) {
  if (n_obs < 0 || n_points < 0) return set_error(HG_ERR_INVALID, "bad sizes");
  if (n_obs > 0 && (!obs_1 || !obs_2 || !obs_3 || !out))
    return set_error(HG_ERR_INVALID, "null pointer");
  if (n_points > 0 && (!pts_1 || !pts_2 || !pts_3 || !coefs))
    return set_error(HG_ERR_INVALID, "null points pointer");
  cudaStream_t st = (cudaStream_t)stream;
  if (spherical)
    return launch_point<1>(kPotential, obs_1, obs_2, obs_3, n_obs, pts_1, pts_2, pts_3, coefs,
                           n_points, out, workspace, workspace_bytes, st, true);
  return launch_point<0>(kPotential, obs_1, obs_2, obs_3, n_obs, pts_1, pts_2, pts_3, coefs,
                         n_points, out, workspace, workspace_bytes, st, true);
}

}  // extern "C"
