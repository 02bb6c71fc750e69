// Magnetic field of uniformly magnetized right-rectangular prisms
// (harmonica src/harmonica/_forward/prisms/magnetic.py, prism_magnetic
// :28-136 and the loops :275-400).
//
// Physics: the scalar potential of a magnetization M is
// phi = -(1/4 pi) M . grad U with U = int 1/R dV, so outside the body
//   b = mu0 H = (mu0 / 4 pi) T M,   T_ab = d2U / dx_a dx_b,
// the gravity gradient tensor kernel of a unit-density prism (no G).  T is
// evaluated with the edge/face formulation of prism_math.cuh (6 face angles,
// 3 merged edge logs per pair).  Outputs in nT (1e9 T).
#include <cuda_runtime.h>

#include <string>

#include "../../include/harmonica_gb300.h"
#include "forward_core.cuh"

namespace hg {

int set_error(int code, const std::string& msg);
int cuda_check(cudaError_t e, const char* what);

namespace {

constexpr double kMu0Over4Pi = 1e-7;  // T m / A

struct MagTile {
  double w[kTile], e[kTile], s[kTile], n[kTile], b[kTile], t[kTile];
  double me[kTile], mn[kTile], mu[kTile];
  int null[kTile];
};

// COMP: 0 b_e, 1 b_n, 2 b_u, 3 all three (rows e, n, u)
template <int COMP>
#ifndef HG_MAG_MIN_BLOCKS
#define HG_MAG_MIN_BLOCKS 4
#endif
__global__ void __launch_bounds__(kThreads, HG_MAG_MIN_BLOCKS) magnetic_kernel(
    const double* __restrict__ oe, const double* __restrict__ on, const double* __restrict__ ou,
    int64_t n_obs, const double* __restrict__ soa, int64_t stride, int64_t n_prisms,
    int64_t chunk, double* __restrict__ dst, int64_t dst_chunk_stride, int scale_output) {
  __shared__ MagTile sh;
  __shared__ SmemTables tabs;
  const Tables T = tabs.stage();
  const int64_t i = (int64_t)blockIdx.x * kThreads + threadIdx.x;
  const bool active = i < n_obs;
  const double pe = active ? oe[i] : 0.0, pn = active ? on[i] : 0.0, pu = active ? ou[i] : 0.0;
  double be = 0.0, bn = 0.0, bu = 0.0;
  const int64_t p0 = (int64_t)blockIdx.y * chunk;
  const int64_t p1 = min(p0 + chunk, n_prisms);
  for (int64_t base = p0; base < p1; base += kTile) {
    const int cnt = (int)min((int64_t)kTile, p1 - base);
    __syncthreads();
    if ((int)threadIdx.x < cnt) {
      const int64_t p = base + threadIdx.x;
      const double w = soa[p], e = soa[stride + p], s = soa[2 * stride + p];
      const double n = soa[3 * stride + p], b = soa[4 * stride + p], t = soa[5 * stride + p];
      const double me = soa[6 * stride + p], mn = soa[7 * stride + p], mu = soa[8 * stride + p];
      sh.w[threadIdx.x] = w;
      sh.e[threadIdx.x] = e;
      sh.s[threadIdx.x] = s;
      sh.n[threadIdx.x] = n;
      sh.b[threadIdx.x] = b;
      sh.t[threadIdx.x] = t;
      sh.me[threadIdx.x] = me;
      sh.mn[threadIdx.x] = mn;
      sh.mu[threadIdx.x] = mu;
      // magnetic.py:430-436: zero volume or null magnetization
      sh.null[threadIdx.x] = (w == e) || (s == n) || (b == t) ||
                             (me == 0.0 && mn == 0.0 && mu == 0.0);
    }
    __syncthreads();
    for (int p = 0; p < cnt; p++) {
      if (sh.null[p]) continue;  // uniform across the CTA
      Rel q;
      q.x1 = sh.w[p] - pe;
      q.x2 = sh.e[p] - pe;
      q.y1 = sh.s[p] - pn;
      q.y2 = sh.n[p] - pn;
      q.z1 = sh.b[p] - pu;
      q.z2 = sh.t[p] - pu;
      q.dx = sh.e[p] - sh.w[p];
      q.dy = sh.n[p] - sh.s[p];
      q.dz = sh.t[p] - sh.b[p];
      const double me = sh.me[p], mn = sh.mn[p], mu = sh.mu[p];
      double t6[6];
      pair_tensor6<true>(q, T, t6);  // ee nn uu en eu nu
      if (COMP == 0 || COMP == 3) be += fma(t6[0], me, fma(t6[3], mn, t6[4] * mu));
      if (COMP == 1 || COMP == 3) bn += fma(t6[3], me, fma(t6[1], mn, t6[5] * mu));
      if (COMP == 2 || COMP == 3) bu += fma(t6[4], me, fma(t6[5], mn, t6[2] * mu));
    }
  }
  if (!active) return;
  const double sc = scale_output ? kMu0Over4Pi * 1e9 : 1.0;
  double* d = dst + (int64_t)blockIdx.y * dst_chunk_stride;
  if (COMP == 3) {
    d[i] = be * sc;
    d[n_obs + i] = bn * sc;
    d[2 * n_obs + i] = bu * sc;
  } else {
    d[i] = (COMP == 0 ? be : (COMP == 1 ? bn : bu)) * sc;
  }
}

__global__ void pack_magnetic_kernel(const double* __restrict__ aos, const double* __restrict__ me,
                                     const double* __restrict__ mn, const double* __restrict__ mu,
                                     int64_t n, double* __restrict__ soa, int64_t stride) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
#pragma unroll
  for (int c = 0; c < 6; c++) soa[c * stride + p] = aos[6 * p + c];
  soa[6 * stride + p] = me[p];
  soa[7 * stride + p] = mn[p];
  soa[8 * stride + p] = mu[p];
}

struct MagPlan {
  int64_t tiles, n_chunks, chunk;
  int rows;
  size_t bytes;
};

MagPlan mag_plan(int64_t n_obs, int64_t n_prisms, int comp) {
  MagPlan p;
  p.rows = comp == 3 ? 3 : 1;
  p.tiles = (n_obs + kThreads - 1) / kThreads;
  const int64_t target = (int64_t)kSmCount * HG_MAG_MIN_BLOCKS * launch_waves();
  int64_t pt = (n_prisms + kTile - 1) / kTile;
  if (pt < 1) pt = 1;
  int64_t want = (target + (p.tiles > 0 ? p.tiles : 1) - 1) / (p.tiles > 0 ? p.tiles : 1);
  want = want < 1 ? 1 : (want > pt ? pt : want);
  if (want > 65535) want = 65535;
  p.chunk = ((pt + want - 1) / want) * kTile;
  p.n_chunks = n_prisms > 0 ? (n_prisms + p.chunk - 1) / p.chunk : 1;
  p.bytes = p.n_chunks > 1 ? (size_t)p.n_chunks * p.rows * (size_t)n_obs * sizeof(double) : 0;
  return p;
}

}  // namespace
}  // namespace hg

using namespace hg;

extern "C" {

int hg_pack_prisms_magnetic(const double* prisms_aos, const double* mag_e, const double* mag_n,
                            const double* mag_u, int64_t n_prisms, double* soa,
                            int64_t prism_stride, void* stream) {
  if (n_prisms < 0 || prism_stride < n_prisms) return set_error(HG_ERR_INVALID, "bad sizes");
  if (n_prisms == 0) return HG_OK;
  if (!prisms_aos || !mag_e || !mag_n || !mag_u || !soa)
    return set_error(HG_ERR_INVALID, "null pointer");
  pack_magnetic_kernel<<<(unsigned)((n_prisms + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
      prisms_aos, mag_e, mag_n, mag_u, n_prisms, soa, prism_stride);
  return cuda_check(cudaGetLastError(), "pack_magnetic_kernel launch");
}

int hg_prism_magnetic_workspace(int64_t n_obs, int64_t n_prisms, int32_t component,
                                size_t* bytes) {
  if (!bytes || n_obs < 0 || n_prisms < 0 || component < 0 || component > 3)
    return set_error(HG_ERR_INVALID, "bad arguments");
  *bytes = mag_plan(n_obs, n_prisms, component).bytes;
  return HG_OK;
}

int hg_prism_magnetic(const double* obs_e, const double* obs_n, const double* obs_u,
                      int64_t n_obs, const double* prisms_soa, int64_t prism_stride,
                      int64_t n_prisms, int32_t component, double* out, void* workspace,
                      size_t workspace_bytes, void* stream) {
  if (n_obs < 0 || n_prisms < 0 || prism_stride < n_prisms || component < 0 || component > 3)
    return set_error(HG_ERR_INVALID, "bad sizes or component");
  if (n_obs > 0 && (!obs_e || !obs_n || !obs_u || !out))
    return set_error(HG_ERR_INVALID, "null pointer");
  if (n_prisms > 0 && !prisms_soa) return set_error(HG_ERR_INVALID, "null prisms pointer");
  cudaStream_t st = (cudaStream_t)stream;
  const MagPlan plan = mag_plan(n_obs, n_prisms, component);
  if (n_obs == 0) return HG_OK;
  if (n_prisms == 0)
    return cuda_check(cudaMemsetAsync(out, 0, sizeof(double) * plan.rows * n_obs, st),
                      "cudaMemsetAsync");
  const bool direct = plan.n_chunks == 1;
  if (!direct && (!workspace || workspace_bytes < plan.bytes))
    return set_error(HG_ERR_INVALID, "workspace missing or too small");
  double* dst = direct ? out : static_cast<double*>(workspace);
  const int64_t cstride = (int64_t)plan.rows * n_obs;
  dim3 grid((unsigned)plan.tiles, (unsigned)plan.n_chunks);
  const int sc = direct ? 1 : 0;
  switch (component) {
    case 0: magnetic_kernel<0><<<grid, kThreads, 0, st>>>(obs_e, obs_n, obs_u, n_obs, prisms_soa, prism_stride, n_prisms, plan.chunk, dst, cstride, sc); break;
    case 1: magnetic_kernel<1><<<grid, kThreads, 0, st>>>(obs_e, obs_n, obs_u, n_obs, prisms_soa, prism_stride, n_prisms, plan.chunk, dst, cstride, sc); break;
    case 2: magnetic_kernel<2><<<grid, kThreads, 0, st>>>(obs_e, obs_n, obs_u, n_obs, prisms_soa, prism_stride, n_prisms, plan.chunk, dst, cstride, sc); break;
    default: magnetic_kernel<3><<<grid, kThreads, 0, st>>>(obs_e, obs_n, obs_u, n_obs, prisms_soa, prism_stride, n_prisms, plan.chunk, dst, cstride, sc); break;
  }
  int rc = cuda_check(cudaGetLastError(), "magnetic_kernel launch");
  if (rc != HG_OK || direct) return rc;
  const int64_t total = cstride;
  launch_chunk_sum(dst, plan.n_chunks, cstride, total, kMu0Over4Pi * 1e9, out, st);
  return cuda_check(cudaGetLastError(), "chunk_sum_kernel launch");
}

}  // extern "C"
