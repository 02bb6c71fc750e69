// All-pairs prism gravity forward kernels and their C ABI (see
// include/harmonica_gb300.h).
//
// Work decomposition: one thread owns one observation point and keeps its
// running sums in registers; a CTA owns a tile of kThreads points and walks a
// CHUNK of the prism list, staged kTile prisms at a time in shared memory as
// structure-of-arrays (every lane of a warp reads the same prism: a broadcast,
// no bank conflicts).  The grid is (point tiles) x (prism chunks); with more
// than one chunk each CTA writes its partial sums to a workspace and a second
// kernel adds the chunks in fixed order, so results do not depend on
// scheduling.  The arithmetic is FP64 throughout.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/harmonica_gb300.h"
#include "forward_core.cuh"

namespace hg {

thread_local std::string g_last_error;

int set_error(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

int cuda_check(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return HG_OK;
  return set_error(HG_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

// out_mask: for kAll, which of the ten fields are written (compact rows).
// PART (accumulate()): 0 writes the whole sums; 1 writes the edge-log part
// (and the pairs taken whole); 2 adds the face part to what part 1 wrote.
template <int F, class Source, int PART = 0>
__global__ void __launch_bounds__(kThreads, PartMinBlocks<F, PART>::value) forward_kernel(
    const double* __restrict__ oe, const double* __restrict__ on, const double* __restrict__ ou,
    int64_t n_obs, Source src, int64_t n_prisms, int64_t chunk, uint32_t out_mask,
    double* __restrict__ dst, int64_t dst_chunk_stride, int scale_output, int check_singular,
    int32_t* __restrict__ flag) {
  constexpr int NF = NumOut<F>::value;
  __shared__ SmemTile sh;
  __shared__ SmemTables tabs;
  const Tables T = tabs.stage();  // made visible by the first barrier in accumulate()

  const int64_t i = (int64_t)blockIdx.x * kThreads + threadIdx.x;
  const bool active = i < n_obs;
  const double pe = active ? oe[i] : 0.0;
  const double pn = active ? on[i] : 0.0;
  const double pu = active ? ou[i] : 0.0;

  // the fused kernel's ten sums in shared memory: they change once per
  // prism tile (the pairs go to float-pair sums), and in registers they
  // would hold 20 of the 128 through the whole pair evaluation
  constexpr bool kSmemAcc = F == kAll;
  double racc[kSmemAcc ? 1 : NF];
  __shared__ double sacc[kSmemAcc ? kThreads * NF : 1];
  double* acc = kSmemAcc ? &sacc[threadIdx.x * NF] : racc;
#pragma unroll
  for (int f = 0; f < NF; f++) acc[f] = 0.0;
  bool singular_seen = false;
  const uint32_t sing_mask = F == kAll ? out_mask : (1u << (F < kNumFields ? F : 0));
  const int64_t p0 = (int64_t)blockIdx.y * chunk;
  const int64_t p1 = min(p0 + chunk, n_prisms);
  accumulate<F, Source, kTile, PART>(src, p0, p1, pe, pn, pu, active, check_singular != 0,
                                     sing_mask, sh, T, acc, singular_seen);
  if (singular_seen) atomicOr(flag, 1);
  if (!active) return;
  double* d = dst + (int64_t)blockIdx.y * dst_chunk_stride;
  if (F == kAll) {
    int row = 0;
#pragma unroll
    for (int f = 0; f < kNumFields; f++) {
      if ((out_mask >> f) & 1u) {
        const double v = scale_output ? acc[f] * field_scale(f) : acc[f];
        double* o = d + (int64_t)row * n_obs + i;
        *o = PART == 2 ? *o + v : v;
        row++;
      }
    }
  } else {
    const double v = scale_output ? acc[0] * field_scale(F) : acc[0];
    d[i] = PART == 2 ? d[i] + v : v;
  }
}

struct RowFields {
  int f[kNumFields];
};

// out[row][i] = scale(field of row) * sum_c part[c][row][i], chunks in order.
// 32 outputs per block: thread (x, y) adds chunks y, y + 16, ... of output x
// (coalesced rows), then the 16 group sums are added in order of y -- a
// fixed order for a given chunk count (deterministic), and 16x the memory
// parallelism of one thread walking all chunks.
constexpr int kReduceGroups = 16;

__global__ void __launch_bounds__(32 * kReduceGroups) reduce_chunks_kernel(
    const double* __restrict__ part, int64_t n_chunks, int64_t chunk_stride, int64_t n_obs,
    int n_rows, RowFields row_field, double* __restrict__ out) {
  __shared__ double group[kReduceGroups][32];
  const int64_t idx = (int64_t)blockIdx.x * 32 + threadIdx.x;
  const int64_t total = (int64_t)n_rows * n_obs;
  double s = 0.0;
  if (idx < total)
    for (int64_t c = threadIdx.y; c < n_chunks; c += kReduceGroups) s += part[c * chunk_stride + idx];
  group[threadIdx.y][threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.y == 0 && idx < total) {
    double t = 0.0;
#pragma unroll
    for (int g = 0; g < kReduceGroups; g++) t += group[g][threadIdx.x];
    out[idx] = t * field_scale(row_field.f[(int)(idx / n_obs)]);
  }
}

// top/bottom of a layer from surface and reference (layer.py:264-312): the
// surface is the top where it is not below the reference; a NaN surface
// compares false and stays the top, with the reference as the bottom.
__global__ void layer_top_bottom_kernel(const double* __restrict__ surface,
                                        const double* __restrict__ reference, double ref_scalar,
                                        int64_t n, double* __restrict__ top,
                                        double* __restrict__ bottom) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double s = surface[i];
  const double r = reference ? reference[i] : ref_scalar;
  const bool reverse = s < r;
  top[i] = reverse ? r : s;
  bottom[i] = reverse ? s : r;
}

__global__ void pack_prisms_kernel(const double* __restrict__ aos, const double* __restrict__ rho,
                                   int64_t n, double* __restrict__ soa, int64_t stride) {
  int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
#pragma unroll
  for (int c = 0; c < 6; c++) soa[c * stride + p] = aos[6 * p + c];
  soa[6 * stride + p] = rho[p];
}

// ---------------------------------------------------------------------------
struct Plan {
  int64_t n_tiles;   // observation tiles (grid.x)
  int64_t n_chunks;  // prism chunks (grid.y)
  int64_t chunk;     // prisms per chunk (multiple of kTile)
  int n_rows;        // output rows
  bool all;          // fused all-field kernel
  int single_field;  // when !all
  size_t workspace_bytes;
};

int popcount10(uint32_t m) {
  int c = 0;
  for (int f = 0; f < kNumFields; f++) c += (m >> f) & 1u;
  return c;
}

Plan make_plan(int64_t n_obs, int64_t n_prisms, uint32_t mask) {
  Plan p;
  p.n_rows = popcount10(mask);
  p.all = p.n_rows != 1;
  p.single_field = -1;
  if (!p.all)
    for (int f = 0; f < kNumFields; f++)
      if ((mask >> f) & 1u) p.single_field = f;
  p.n_tiles = (n_obs + kThreads - 1) / kThreads;
  // Enough CTAs for many full waves of the resident CTAs on every SM
  // (launch_waves()); split the prisms when the observation tiles alone
  // cannot fill the GPU.  Measured on the g_z bench step (5000 stations x
  // 1e6 prisms): 1 wave 1.09e10 pairs/s, 2 1.14e10, 4 1.18e10, 16 1.20e10,
  // 32 1.21e10 (the old fixed 8 CTAs per SM was 1.6 waves).
  const bool wide = p.all || p.single_field == kPotential;
  const bool grad = p.single_field == kGe || p.single_field == kGn || p.single_field == kGz;
  const int64_t resident =
      wide ? HG_FWD_MIN_BLOCKS_PART : (grad ? HG_FWD_MIN_BLOCKS_GRAD : HG_FWD_MIN_BLOCKS);
  const int64_t target = (int64_t)kSmCount * resident * launch_waves();
  int64_t n_prism_tiles = (n_prisms + kTile - 1) / kTile;
  if (n_prism_tiles < 1) n_prism_tiles = 1;
  int64_t want = (target + p.n_tiles - 1) / p.n_tiles;
  if (want < 1) want = 1;
  if (want > n_prism_tiles) want = n_prism_tiles;
  if (want > 65535) want = 65535;
  int64_t tiles_per_chunk = (n_prism_tiles + want - 1) / want;
  p.chunk = tiles_per_chunk * kTile;
  p.n_chunks = (n_prisms + p.chunk - 1) / p.chunk;
  if (p.n_chunks < 1) p.n_chunks = 1;
  p.workspace_bytes =
      p.n_chunks > 1 ? (size_t)p.n_chunks * p.n_rows * n_obs * sizeof(double) : 0;
  return p;
}

// The plan with at most as many prism chunks as `max_bytes` of partial sums
// hold: longer chunks (a whole number of tiles) when the plan's own chunking
// needs more, one chunk (no partial sums at all) when fewer than two fit.
Plan cap_plan(Plan p, int64_t n_obs, int64_t n_prisms, size_t max_bytes) {
  if (p.workspace_bytes <= max_bytes) return p;
  const size_t per_chunk = (size_t)p.n_rows * (size_t)n_obs * sizeof(double);
  const int64_t max_chunks = (int64_t)(max_bytes / per_chunk);
  int64_t n_prism_tiles = (n_prisms + kTile - 1) / kTile;
  if (n_prism_tiles < 1) n_prism_tiles = 1;
  const int64_t tiles_per_chunk =
      max_chunks < 2 ? n_prism_tiles : (n_prism_tiles + max_chunks - 1) / max_chunks;
  p.chunk = tiles_per_chunk * kTile;
  p.n_chunks = (n_prisms + p.chunk - 1) / p.chunk;
  if (p.n_chunks < 1) p.n_chunks = 1;
  p.workspace_bytes = p.n_chunks > 1 ? (size_t)p.n_chunks * per_chunk : 0;
  return p;
}

template <class Source>
int launch_forward(const Plan& plan, const double* oe, const double* on, const double* ou,
                   int64_t n_obs, const Source& src, int64_t n_prisms, uint32_t mask, double* out,
                   int32_t* flag, void* workspace, cudaStream_t stream, bool check_singular) {
  if (n_obs == 0) return HG_OK;
  if (plan.n_tiles > 2147483647LL) return set_error(HG_ERR_INVALID, "too many observation points");
  const bool direct = plan.n_chunks == 1;
  double* dst = out;
  int64_t chunk_stride = 0;
  // A workspace this call allocated itself is released on every return path.
  struct OwnedWorkspace {
    void* ptr = nullptr;
    cudaStream_t stream = nullptr;
    ~OwnedWorkspace() {
      if (ptr) cudaFreeAsync(ptr, stream);
    }
  } owned;
  if (!direct) {
    if (workspace == nullptr) {
      cudaError_t e = cudaMallocAsync(&workspace, plan.workspace_bytes, stream);
      if (e != cudaSuccess) return cuda_check(e, "cudaMallocAsync(workspace)");
      owned.ptr = workspace;
      owned.stream = stream;
    }
    dst = static_cast<double*>(workspace);
    chunk_stride = (int64_t)plan.n_rows * n_obs;
  }
  if (n_prisms == 0)
    return cuda_check(cudaMemsetAsync(out, 0, sizeof(double) * plan.n_rows * n_obs, stream),
                      "cudaMemsetAsync(out)");
  if (flag == nullptr) check_singular = false;
  dim3 grid((unsigned)plan.n_tiles, (unsigned)plan.n_chunks);
  const int scale = direct ? 1 : 0;
  const int cs = check_singular ? 1 : 0;
  int32_t* fl = flag;
  if (plan.all || plan.single_field == kPotential) {
    // edge-log part, then face part added in place (same stream: ordered)
    if (plan.all) {
      forward_kernel<kAll, Source, 1><<<grid, kThreads, 0, stream>>>(
          oe, on, ou, n_obs, src, n_prisms, plan.chunk, mask, dst, chunk_stride, scale, cs, fl);
      forward_kernel<kAll, Source, 2><<<grid, kThreads, 0, stream>>>(
          oe, on, ou, n_obs, src, n_prisms, plan.chunk, mask, dst, chunk_stride, scale, 0, fl);
    } else {
      forward_kernel<kPotential, Source, 1><<<grid, kThreads, 0, stream>>>(
          oe, on, ou, n_obs, src, n_prisms, plan.chunk, mask, dst, chunk_stride, scale, cs, fl);
      forward_kernel<kPotential, Source, 2><<<grid, kThreads, 0, stream>>>(
          oe, on, ou, n_obs, src, n_prisms, plan.chunk, mask, dst, chunk_stride, scale, 0, fl);
    }
  } else {
    switch (plan.single_field) {
#define HG_CASE(FF)                                                                            \
  case FF:                                                                                     \
    forward_kernel<FF, Source><<<grid, kThreads, 0, stream>>>(oe, on, ou, n_obs, src, n_prisms, \
                                                             plan.chunk, mask, dst,            \
                                                             chunk_stride, scale, cs, fl);     \
    break;
      HG_CASE(1) HG_CASE(2) HG_CASE(3) HG_CASE(4)
      HG_CASE(5) HG_CASE(6) HG_CASE(7) HG_CASE(8) HG_CASE(9)
#undef HG_CASE
      default: return set_error(HG_ERR_INVALID, "bad field");
    }
  }
  int rc = cuda_check(cudaGetLastError(), "forward_kernel launch");
  if (rc != HG_OK) return rc;
  if (!direct) {
    RowFields rf{};
    int r = 0;
    for (int f = 0; f < kNumFields; f++)
      if ((mask >> f) & 1u) rf.f[r++] = f;
    int64_t total = (int64_t)plan.n_rows * n_obs;
    int64_t blocks = (total + 31) / 32;
    reduce_chunks_kernel<<<(unsigned)blocks, dim3(32, kReduceGroups), 0, stream>>>(
        dst, plan.n_chunks, chunk_stride, n_obs, plan.n_rows, rf, out);
    rc = cuda_check(cudaGetLastError(), "reduce_chunks_kernel launch");
    if (rc != HG_OK) return rc;
  }
  return HG_OK;
}

bool valid_mask(uint32_t m) { return m != 0 && (m & ~HG_FIELD_MASK_ALL) == 0; }

}  // namespace hg

using namespace hg;

extern "C" {

int hg_version(void) { return 100; }

const char* hg_last_error(void) { return g_last_error.c_str(); }

int hg_pack_prisms(const double* prisms_aos, const double* density, int64_t n_prisms,
                   double* prisms_soa, int64_t prism_stride, void* stream) {
  if (n_prisms < 0 || prism_stride < n_prisms) return set_error(HG_ERR_INVALID, "bad sizes");
  if (n_prisms == 0) return HG_OK;
  if (!prisms_aos || !density || !prisms_soa) return set_error(HG_ERR_INVALID, "null pointer");
  int threads = 256;
  int64_t blocks = (n_prisms + threads - 1) / threads;
  pack_prisms_kernel<<<(unsigned)blocks, threads, 0, (cudaStream_t)stream>>>(
      prisms_aos, density, n_prisms, prisms_soa, prism_stride);
  return cuda_check(cudaGetLastError(), "pack_prisms_kernel launch");
}

int hg_layer_top_bottom(const double* surface, const double* reference, double reference_value,
                        int64_t n, double* top, double* bottom, void* stream) {
  if (n < 0) return set_error(HG_ERR_INVALID, "bad size");
  if (n == 0) return HG_OK;
  if (!surface || !top || !bottom) return set_error(HG_ERR_INVALID, "null pointer");
  const int threads = 256;
  const int64_t blocks = (n + threads - 1) / threads;
  layer_top_bottom_kernel<<<(unsigned)blocks, threads, 0, (cudaStream_t)stream>>>(
      surface, reference, reference_value, n, top, bottom);
  return cuda_check(cudaGetLastError(), "layer_top_bottom_kernel launch");
}

int hg_prism_forward_workspace(int64_t n_obs, int64_t n_prisms, uint32_t field_mask,
                               size_t* bytes) {
  if (!bytes) return set_error(HG_ERR_INVALID, "null pointer");
  if (n_obs < 0 || n_prisms < 0 || !valid_mask(field_mask))
    return set_error(HG_ERR_INVALID, "bad sizes or field mask");
  *bytes = make_plan(n_obs, n_prisms, field_mask).workspace_bytes;
  return HG_OK;
}

int hg_prism_forward(const double* obs_e, const double* obs_n, const double* obs_u, int64_t n_obs,
                     const double* prisms_soa, int64_t prism_stride, int64_t n_prisms,
                     uint32_t field_mask, double* out, int32_t* singular_flag, void* workspace,
                     size_t workspace_bytes, void* stream) {
  if (n_obs < 0 || n_prisms < 0 || prism_stride < n_prisms || !valid_mask(field_mask))
    return set_error(HG_ERR_INVALID, "bad sizes or field mask");
  if (n_obs > 0 && (!obs_e || !obs_n || !obs_u || !out))
    return set_error(HG_ERR_INVALID, "null pointer");
  if (n_prisms > 0 && !prisms_soa) return set_error(HG_ERR_INVALID, "null prisms pointer");
  Plan plan = make_plan(n_obs, n_prisms, field_mask);
  if (workspace && workspace_bytes < plan.workspace_bytes)
    return set_error(HG_ERR_INVALID, "workspace too small");
  ListSource src{prisms_soa, prism_stride};
  return launch_forward(plan, obs_e, obs_n, obs_u, n_obs, src, n_prisms, field_mask, out,
                        singular_flag, workspace, (cudaStream_t)stream, true);
}

int hg_layer_forward_workspace(int64_t n_obs, int64_t n_east, int64_t n_north,
                               uint32_t field_mask, size_t* bytes) {
  if (!bytes) return set_error(HG_ERR_INVALID, "null pointer");
  if (n_obs < 0 || n_east < 0 || n_north < 0 || !valid_mask(field_mask))
    return set_error(HG_ERR_INVALID, "bad sizes or field mask");
  *bytes = make_plan(n_obs, n_east * n_north, field_mask).workspace_bytes;
  return HG_OK;
}

int hg_layer_forward(const double* obs_e, const double* obs_n, const double* obs_u, int64_t n_obs,
                     const double* centre_e, int64_t n_east, const double* centre_n,
                     int64_t n_north, const double* bottom, const double* top,
                     const double* density, double thickness_threshold, uint32_t field_mask,
                     double* out, void* workspace, size_t workspace_bytes, void* stream) {
  if (n_obs < 0 || n_east < 2 || n_north < 2 || !valid_mask(field_mask))
    return set_error(HG_ERR_INVALID, "bad sizes or field mask (layer needs >= 2 x 2 prisms)");
  if (n_obs > 0 && (!obs_e || !obs_n || !obs_u || !out))
    return set_error(HG_ERR_INVALID, "null pointer");
  if (!centre_e || !centre_n || !bottom || !top || !density)
    return set_error(HG_ERR_INVALID, "null layer pointer");
  cudaStream_t st = (cudaStream_t)stream;
  int64_t n_prisms = n_east * n_north;
  Plan plan = make_plan(n_obs, n_prisms, field_mask);
  if (workspace && workspace_bytes < plan.workspace_bytes)
    return set_error(HG_ERR_INVALID, "workspace too small");
  LayerSource src{centre_e, centre_n, bottom, top, density, n_east, thickness_threshold};
  return launch_forward(plan, obs_e, obs_n, obs_u, n_obs, src, n_prisms, field_mask, out, nullptr,
                        workspace, st, false);
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Forward for callers that cannot allocate device memory.
//
// Who needs this: code running under a host framework that owns the device
// memory pool and forbids foreign cudaMalloc calls; latency-critical loops
// where an allocation (with its possible implicit synchronisation, or its
// failure under memory pressure) is not acceptable in the middle of a step;
// and plugins whose GPU memory budget is fixed when the process starts.
// hg_prism_forward needs scratch space for per-chunk partial sums whenever
// the observation points alone cannot fill the GPU, and such a caller can
// neither hand it a workspace nor let it call cudaMallocAsync.
// hg_prism_forward_noalloc runs the same kernels with that scratch taken from
// a fixed array compiled into the library (kNoAllocScratchBytes = 8 MiB; every
// GPU that loads the library holds it until the process exits).  Problems
// whose usual chunking would need more partial sums than the array holds run
// with fewer, longer chunks (cap_plan), down to one chunk, which needs no
// scratch; so no problem is rejected for its size, and the only cost is less
// parallelism for many fields at once over tens of thousands of points.

namespace {

constexpr size_t kNoAllocScratchBytes = size_t(8) << 20;
constexpr int kNoAllocMaxDevices = 64;

}  // namespace

// The scratch array.  In host code its name is only a host-side stand-in, so
// its device address is looked up once per device (see noalloc_scratch).
static __device__ __align__(256) double g_noalloc_scratch[kNoAllocScratchBytes / sizeof(double)];

namespace {

std::mutex g_noalloc_mutex;
double* g_noalloc_ptr[kNoAllocMaxDevices] = {};

// Device address of g_noalloc_scratch on the current device, looked up with
// cudaGetSymbolAddress the first time each device is used and kept for the
// life of the process (a device reset while the library is in use would
// leave it stale: callers must not reset a device they use this entry on).
int noalloc_scratch(double** ptr) {
  int dev = 0;
  int rc = cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
  if (rc != HG_OK) return rc;
  if (dev < 0 || dev >= kNoAllocMaxDevices)
    return set_error(HG_ERR_INVALID, "hg_prism_forward_noalloc: device index out of range");
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (g_noalloc_ptr[dev] == nullptr) {
    void* p = nullptr;
    rc = cuda_check(cudaGetSymbolAddress(&p, g_noalloc_scratch),
                    "cudaGetSymbolAddress(no-alloc scratch)");
    if (rc != HG_OK) return rc;
    g_noalloc_ptr[dev] = static_cast<double*>(p);
  }
  *ptr = g_noalloc_ptr[dev];
  return HG_OK;
}

}  // namespace

extern "C" int hg_prism_forward_noalloc(const double* obs_e, const double* obs_n,
                                        const double* obs_u, int64_t n_obs,
                                        const double* prisms_soa, int64_t prism_stride,
                                        int64_t n_prisms, uint32_t field_mask, double* out,
                                        int32_t* singular_flag, void* stream) {
  if (n_obs < 0 || n_prisms < 0 || prism_stride < n_prisms || !valid_mask(field_mask))
    return set_error(HG_ERR_INVALID, "bad sizes or field mask");
  if (n_obs > 0 && (!obs_e || !obs_n || !obs_u || !out))
    return set_error(HG_ERR_INVALID, "null pointer");
  if (n_prisms > 0 && !prisms_soa) return set_error(HG_ERR_INVALID, "null prisms pointer");
  const Plan plan =
      cap_plan(make_plan(n_obs, n_prisms, field_mask), n_obs, n_prisms, kNoAllocScratchBytes);
  // cap_plan keeps every plan within the array; this check guards that invariant
  if (plan.workspace_bytes > kNoAllocScratchBytes)
    return set_error(HG_ERR_INVALID,
                     "hg_prism_forward_noalloc: this problem needs " +
                         std::to_string(plan.workspace_bytes) +
                         " bytes of scratch, more than the fixed " +
                         std::to_string(kNoAllocScratchBytes) + " bytes");
  double* scratch = nullptr;
  if (plan.workspace_bytes > 0) {
    const int rc = noalloc_scratch(&scratch);
    if (rc != HG_OK) return rc;
  }
  // Every partial-sum slot the reduction reads is written by the forward
  // launch first, so the scratch left by an earlier call needs no clearing.
  ListSource src{prisms_soa, prism_stride};
  return launch_forward(plan, obs_e, obs_n, obs_u, n_obs, src, n_prisms, field_mask, out,
                        singular_flag, scratch, (cudaStream_t)stream, true);
}
