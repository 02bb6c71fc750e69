// Adjoint (transpose) of the prism forward, for gradients of a misfit.
//
// With d_i = sum_j rho_j K_f(x_i; prism_j) (field f, harmonica units) and
// weights w_i = dL/dd_i, the adjoint returns
//   dL/drho_j    = sum_i w_i K_f(x_i; prism_j)                (any field)
//   dL/dbottom_j = rho_j sum_i w_i dK_gz/dbottom = rho_j G 1e5 sum_i w_i O_bottom,ij
//   dL/dtop_j    = -rho_j G 1e5 sum_i w_i O_top,ij              (g_z only)
// where O is the face angle of the prism's horizontal face seen from point i
// (the closed-form face integral of the g_z kernel; see pair_gz_faces).
//
// Work decomposition: the transpose of the forward kernels -- one thread owns
// one prism (kept in registers) and the CTA walks a chunk of the points,
// staged with their weights in shared memory; partial sums per point chunk
// go to a workspace and are added in fixed order.
#include <cuda_runtime.h>

#include <string>

#include "../../include/harmonica_gb300.h"
#include "forward_core.cuh"

namespace hg {

int set_error(int code, const std::string& msg);
int cuda_check(cudaError_t e, const char* what);

namespace {

struct PointTile {
  double e[kTile], n[kTile], u[kTile], w[kTile];
};

constexpr int kAdjOut = 3;  // density, bottom, top

#ifndef HG_ADJ_MIN_BLOCKS
#define HG_ADJ_MIN_BLOCKS 4
#endif
// Resident CTAs per SM: the potential's adjoint needs every log and face angle
template <int F> struct AdjMinBlocks { static constexpr int value = HG_ADJ_MIN_BLOCKS; };
template <> struct AdjMinBlocks<kPotential> { static constexpr int value = 3; };

// part layout: [chunk][output][prism]
template <int F, class Source>
__global__ void __launch_bounds__(kThreads, AdjMinBlocks<F>::value) adjoint_kernel(
    const double* __restrict__ oe, const double* __restrict__ on, const double* __restrict__ ou,
    const double* __restrict__ weights, int64_t n_obs, Source src, int64_t n_prisms,
    int64_t chunk, double* __restrict__ part) {
  __shared__ PointTile sh;
  __shared__ SmemTables tabs;
  const Tables T = tabs.stage();
  const int64_t j = (int64_t)blockIdx.x * kThreads + threadIdx.x;
  const bool active = j < n_prisms;
  double w = 0, e = 0, s = 0, n = 0, b = 0, t = 0, rho = 0;
  bool null = true;
  if (active) src.load(j, w, e, s, n, b, t, rho, null);
  double acc_rho = 0.0, acc_b = 0.0, acc_t = 0.0;
  const int64_t i0 = (int64_t)blockIdx.y * chunk;
  const int64_t i1 = min(i0 + chunk, n_obs);
  for (int64_t base = i0; base < i1; base += kTile) {
    const int cnt = (int)min((int64_t)kTile, i1 - base);
    __syncthreads();
    if ((int)threadIdx.x < cnt) {
      sh.e[threadIdx.x] = oe[base + threadIdx.x];
      sh.n[threadIdx.x] = on[base + threadIdx.x];
      sh.u[threadIdx.x] = ou[base + threadIdx.x];
      sh.w[threadIdx.x] = weights[base + threadIdx.x];
    }
    __syncthreads();
    if (null) continue;  // per-thread: this thread's prism contributes nothing
    for (int k = 0; k < cnt; k++) {
      Rel q;
      q.x1 = w - sh.e[k];
      q.x2 = e - sh.e[k];
      q.y1 = s - sh.n[k];
      q.y2 = n - sh.n[k];
      q.z1 = b - sh.u[k];
      q.z2 = t - sh.u[k];
      q.dx = e - w;
      q.dy = n - s;
      q.dz = t - b;
      const double wk = sh.w[k];
      if (F == kGz) {
        double ob, ot;
        const double v = pair_gz_faces<true>(q, T, ob, ot);
        acc_rho = fma(wk, v, acc_rho);
        acc_b = fma(wk, ob, acc_b);
        acc_t = fma(wk, ot, acc_t);
      } else {
        double v = pair_field<F, true>(q, T);
        if (is_tensor(F) && singular_for(F, q)) v = quiet_nan();
        acc_rho = fma(wk, v, acc_rho);
      }
    }
  }
  if (!active) return;
  double* d = part + (int64_t)blockIdx.y * kAdjOut * n_prisms;
  d[j] = acc_rho;
  d[n_prisms + j] = acc_b * rho;
  d[2 * n_prisms + j] = -acc_t * rho;
}

// grad[o][j] = scale * sum_c part[c][o][j]
__global__ void adjoint_reduce_kernel(const double* __restrict__ part, int64_t n_chunks,
                                      int64_t n_prisms, double scale_rho, double scale_geom,
                                      double* __restrict__ g_rho, double* __restrict__ g_bottom,
                                      double* __restrict__ g_top) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n_prisms) return;
  double sr = 0.0, sb = 0.0, st = 0.0;
  for (int64_t c = 0; c < n_chunks; c++) {
    const double* d = part + c * kAdjOut * n_prisms;
    sr += d[j];
    sb += d[n_prisms + j];
    st += d[2 * n_prisms + j];
  }
  if (g_rho) g_rho[j] = sr * scale_rho;
  if (g_bottom) g_bottom[j] = sb * scale_geom;
  if (g_top) g_top[j] = st * scale_geom;
}

struct AdjPlan {
  int64_t tiles, n_chunks, chunk;
  size_t bytes;
};

AdjPlan adj_plan(int64_t n_obs, int64_t n_prisms) {
  AdjPlan p;
  p.tiles = (n_prisms + kThreads - 1) / kThreads;
  const int64_t target = (int64_t)kSmCount * HG_ADJ_MIN_BLOCKS * launch_waves();
  int64_t point_tiles = (n_obs + kTile - 1) / kTile;
  if (point_tiles < 1) point_tiles = 1;
  int64_t want = (target + p.tiles - 1) / (p.tiles > 0 ? p.tiles : 1);
  want = want < 1 ? 1 : (want > point_tiles ? point_tiles : want);
  if (want > 65535) want = 65535;
  p.chunk = ((point_tiles + want - 1) / want) * kTile;
  p.n_chunks = n_obs > 0 ? (n_obs + p.chunk - 1) / p.chunk : 1;
  p.bytes = (size_t)p.n_chunks * kAdjOut * (size_t)n_prisms * sizeof(double);
  return p;
}

template <class Source>
int launch_adjoint(int field, const double* oe, const double* on, const double* ou,
                   const double* wts, int64_t n_obs, const Source& src, int64_t n_prisms,
                   double* g_rho, double* g_bottom, double* g_top, void* workspace,
                   size_t workspace_bytes, cudaStream_t st) {
  if (n_prisms == 0) return HG_OK;
  const AdjPlan plan = adj_plan(n_obs, n_prisms);
  if (!workspace || workspace_bytes < plan.bytes)
    return set_error(HG_ERR_INVALID, "workspace missing or too small");
  if (field != kGz && (g_bottom || g_top))
    return set_error(HG_ERR_INVALID, "bottom/top gradients are available for g_z only");
  double* part = static_cast<double*>(workspace);
  if (n_obs == 0) {
    int rc = cuda_check(cudaMemsetAsync(part, 0, plan.bytes, st), "cudaMemsetAsync");
    if (rc != HG_OK) return rc;
  } else {
    dim3 grid((unsigned)plan.tiles, (unsigned)plan.n_chunks);
    switch (field) {
#define HG_ADJ(FF)                                                                         \
  case FF:                                                                                 \
    adjoint_kernel<FF, Source><<<grid, kThreads, 0, st>>>(oe, on, ou, wts, n_obs, src,     \
                                                         n_prisms, plan.chunk, part);      \
    break;
      HG_ADJ(0) HG_ADJ(1) HG_ADJ(2) HG_ADJ(3) HG_ADJ(4)
      HG_ADJ(5) HG_ADJ(6) HG_ADJ(7) HG_ADJ(8) HG_ADJ(9)
#undef HG_ADJ
      default: return set_error(HG_ERR_INVALID, "bad field");
    }
    int rc = cuda_check(cudaGetLastError(), "adjoint_kernel launch");
    if (rc != HG_OK) return rc;
  }
  const int threads = 256;
  adjoint_reduce_kernel<<<(unsigned)((n_prisms + threads - 1) / threads), threads, 0, st>>>(
      part, n_obs == 0 ? 1 : plan.n_chunks, n_prisms, field_scale(field), kG * 1e5, g_rho,
      g_bottom, g_top);
  return cuda_check(cudaGetLastError(), "adjoint_reduce_kernel launch");
}

}  // namespace
}  // namespace hg

using namespace hg;

extern "C" {

int hg_prism_adjoint_workspace(int64_t n_obs, int64_t n_prisms, size_t* bytes) {
  if (!bytes || n_obs < 0 || n_prisms < 0) return set_error(HG_ERR_INVALID, "bad arguments");
  *bytes = adj_plan(n_obs, n_prisms).bytes;
  return HG_OK;
}

int hg_prism_adjoint(const double* obs_e, const double* obs_n, const double* obs_u,
                     const double* weights, int64_t n_obs, const double* prisms_soa,
                     int64_t prism_stride, int64_t n_prisms, int32_t field, double* grad_density,
                     double* grad_bottom, double* grad_top, void* workspace,
                     size_t workspace_bytes, void* stream) {
  if (n_obs < 0 || n_prisms < 0 || prism_stride < n_prisms || field < 0 || field >= kNumFields)
    return set_error(HG_ERR_INVALID, "bad sizes or field");
  if (n_obs > 0 && (!obs_e || !obs_n || !obs_u || !weights))
    return set_error(HG_ERR_INVALID, "null pointer");
  if (n_prisms > 0 && !prisms_soa) return set_error(HG_ERR_INVALID, "null prisms pointer");
  return launch_adjoint(field, obs_e, obs_n, obs_u, weights, n_obs,
                        ListSource{prisms_soa, prism_stride}, n_prisms, grad_density,
                        grad_bottom, grad_top, workspace, workspace_bytes, (cudaStream_t)stream);
}

int hg_layer_adjoint_workspace(int64_t n_obs, int64_t n_east, int64_t n_north, size_t* bytes) {
  if (!bytes || n_obs < 0 || n_east < 0 || n_north < 0)
    return set_error(HG_ERR_INVALID, "bad arguments");
  *bytes = adj_plan(n_obs, n_east * n_north).bytes;
  return HG_OK;
}

int hg_layer_adjoint(const double* obs_e, const double* obs_n, const double* obs_u,
                     const double* weights, int64_t n_obs, const double* centre_e, int64_t n_east,
                     const double* centre_n, int64_t n_north, const double* bottom,
                     const double* top, const double* density, double thickness_threshold,
                     int32_t field, double* grad_density, double* grad_bottom, double* grad_top,
                     void* workspace, size_t workspace_bytes, void* stream) {
  if (n_obs < 0 || n_east < 2 || n_north < 2 || field < 0 || field >= kNumFields)
    return set_error(HG_ERR_INVALID, "bad sizes or field (layer needs >= 2 x 2 prisms)");
  if (n_obs > 0 && (!obs_e || !obs_n || !obs_u || !weights))
    return set_error(HG_ERR_INVALID, "null pointer");
  if (!centre_e || !centre_n || !bottom || !top || !density)
    return set_error(HG_ERR_INVALID, "null layer pointer");
  LayerSource src{centre_e, centre_n, bottom, top, density, n_east, thickness_threshold};
  return launch_adjoint(field, obs_e, obs_n, obs_u, weights, n_obs, src, n_east * n_north,
                        grad_density, grad_bottom, grad_top, workspace, workspace_bytes,
                        (cudaStream_t)stream);
}

}  // extern "C"
