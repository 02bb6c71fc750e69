// Batched prism forward: many independent (points, prisms, field) problems of
// very different sizes in ONE persistent launch.
//
// The host cuts every problem into work items (problem, point tile of
// kThreads points, prism chunk) and sorts them by decreasing cost.  A
// persistent grid of CTAs pulls items from a device counter (atomicAdd, no
// waiting on other CTAs), so small and large problems share the GPU without
// tail effects.  Each item writes its partial sums into its own slot of a
// workspace and a second kernel adds each point's chunks in fixed order and
// applies the units: results are bitwise independent of the schedule and of
// the other problems in the batch.  hg_batch_run only issues a memset and two
// launches on the caller's stream (no allocation, no host synchronisation),
// so it can be captured in a CUDA graph and replayed.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/harmonica_gb300.h"
#include "batch_core.cuh"

namespace hg {



int set_error(int code, const std::string& msg);
int cuda_check(cudaError_t e, const char* what);

BatchKernel batch_kernel_for(int f, int threads) {
  return threads == 64 ? batch_kernel_for64(f) : batch_kernel_table<kThreads>(f);
}
BatchKernel batch_potential_faces_for(int threads) {
  return threads == 64 ? batch_potential_faces64() : batch_potential_faces<kThreads>();
}

// out_p[i] = scale(field_p) * sum_c part_p[c][i], chunks in order.
__global__ void batch_reduce_kernel(const ProblemDev* __restrict__ probs,
                                    const double* __restrict__ part) {
  const ProblemDev P = probs[blockIdx.y];
  const double scale = field_scale(P.field);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < P.n_obs;
       i += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int64_t c = 0; c < P.n_chunks; c++) s += part[P.part_offset + c * P.n_obs + i];
    P.out[i] = s * scale;
  }
}

}  // namespace hg

using namespace hg;

struct hg_batch {
  int64_t n_problems = 0;
  int64_t n_items = 0;
  int64_t seg_begin[kNumFields] = {};  // the items of field f: [seg_begin, seg_begin + seg_count)
  int64_t seg_count[kNumFields] = {};
  int32_t seg_ctas[kNumFields] = {};   // CTAs of field f's persistent launch
  int32_t seg_threads[kNumFields] = {};  // points per CTA of field f's launch
  int64_t n_ctas = 0;
  int64_t partials = 0;  // doubles
  double pairs = 0.0;
  ProblemDev* d_probs = nullptr;
  WorkItem* d_items = nullptr;
  int device = 0;
};

namespace {

constexpr size_t kCounterBytes = 256;  // one counter per field, then the partials (256-byte aligned)

int64_t round_up(int64_t a, int64_t b) { return (a + b - 1) / b * b; }

}  // namespace

extern "C" {

int hg_batch_create_shaped(const hg_problem* problems, int64_t n_problems,
                           const hg_batch_shape* shapes, hg_batch** batch) {
  if (!batch || !shapes || n_problems < 0 || (n_problems > 0 && !problems))
    return set_error(HG_ERR_INVALID, "bad arguments");
  if (n_problems > 65535) return set_error(HG_ERR_INVALID, "at most 65535 problems per batch");
  *batch = nullptr;
  for (int f = 0; f < kNumFields; f++)
    if (shapes[f].points_per_cta != 0 && shapes[f].points_per_cta != 64 &&
        shapes[f].points_per_cta != 128)
      return set_error(HG_ERR_INVALID, "points_per_cta must be 0, 64 or 128");
  int device = 0;
  int rc = cuda_check(cudaGetDevice(&device), "cudaGetDevice");
  if (rc != HG_OK) return rc;
  int sms = kSmCount;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  // per field: points per CTA, and the CTAs of its persistent launch (the
  // given count, else one full wave of that field's kernel)
  int32_t threads_for[kNumFields], ctas_for[kNumFields];
  for (int f = 0; f < kNumFields; f++) {
    threads_for[f] = shapes[f].points_per_cta > 0 ? shapes[f].points_per_cta : kThreads;
    ctas_for[f] = shapes[f].n_ctas;
    if (ctas_for[f] <= 0) {
      int per_sm = 0;
      rc = cuda_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                          &per_sm, batch_kernel_for(f, threads_for[f]), threads_for[f], 0),
                      "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
      if (rc != HG_OK) return rc;
      ctas_for[f] = (int32_t)std::max(1, per_sm) * sms;
    }
  }
  std::vector<ProblemDev> probs((size_t)n_problems);
  double field_pairs[kNumFields] = {};
  for (int64_t p = 0; p < n_problems; p++) {
    const hg_problem& q = problems[p];
    if (q.n_obs < 0 || q.n_prisms < 0 || q.prism_stride < q.n_prisms || q.field < 0 ||
        q.field >= kNumFields)
      return set_error(HG_ERR_INVALID, "bad problem " + std::to_string(p));
    if (q.n_obs > 0 && (!q.obs_e || !q.obs_n || !q.obs_u || !q.out))
      return set_error(HG_ERR_INVALID, "null pointer in problem " + std::to_string(p));
    if (q.n_prisms > 0 && !q.prisms_soa)
      return set_error(HG_ERR_INVALID, "null prisms in problem " + std::to_string(p));
    field_pairs[q.field] += (double)q.n_obs * (double)q.n_prisms;
  }
  // Chunk size per field: the given one (rounded up to whole prism tiles of
  // that field's CTA shape), else enough items to keep every CTA of the
  // field's launch busy ~16 times over.
  int64_t chunk_for[kNumFields];
  for (int f = 0; f < kNumFields; f++) {
    const int64_t tile = threads_for[f];
    if (shapes[f].chunk_prisms > 0) {
      chunk_for[f] = round_up(shapes[f].chunk_prisms, tile);
    } else {
      const double target_items = 16.0 * ctas_for[f];
      const double pairs_per_item = std::max(1.0, field_pairs[f] / target_items);
      chunk_for[f] = round_up(std::max<int64_t>(tile, (int64_t)(pairs_per_item / tile)), tile);
    }
  }
  std::vector<WorkItem> items;
  std::vector<double> cost;
  int64_t part = 0;
  double pairs = 0.0;
  for (int64_t p = 0; p < n_problems; p++) {
    const hg_problem& q = problems[p];
    ProblemDev& d = probs[(size_t)p];
    d.e = q.obs_e;
    d.n = q.obs_n;
    d.u = q.obs_u;
    d.n_obs = q.n_obs;
    d.soa = q.prisms_soa;
    d.stride = q.prism_stride;
    d.n_prisms = q.n_prisms;
    d.chunk = chunk_for[q.field];
    d.n_chunks = q.n_prisms > 0 ? (q.n_prisms + d.chunk - 1) / d.chunk : 0;
    d.part_offset = part;
    d.out = q.out;
    d.flag = q.singular_flag;
    d.field = q.field;
    d.check_singular = q.check_singular;
    part += d.n_chunks * q.n_obs;
    pairs += (double)q.n_obs * (double)q.n_prisms;
    const int64_t threads = threads_for[q.field];
    const int64_t tiles = (q.n_obs + threads - 1) / threads;
    if (tiles > INT32_MAX || d.n_chunks > INT32_MAX || n_problems > INT32_MAX)
      return set_error(HG_ERR_INVALID, "problem too large for the work list");
    for (int64_t t = 0; t < tiles; t++)
      for (int64_t c = 0; c < d.n_chunks; c++) {
        items.push_back(WorkItem{(int32_t)p, (int32_t)t, (int32_t)c, 0});
        const double np = (double)std::min(d.chunk, q.n_prisms - c * d.chunk);
        cost.push_back(np * (double)threads);  // threads x prisms of the item
      }
  }
  // grouped by field; within a field longest items first (list
  // scheduling), ties in creation order
  std::vector<int64_t> order(items.size());
  for (size_t k = 0; k < order.size(); k++) order[k] = (int64_t)k;
  const auto field_of = [&](int64_t k) { return probs[(size_t)items[(size_t)k].problem].field; };
  std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t b) {
    const int fa = field_of(a), fb = field_of(b);
    if (fa != fb) return fa < fb;
    return cost[(size_t)a] > cost[(size_t)b];
  });
  std::vector<WorkItem> sorted(items.size());
  for (size_t k = 0; k < order.size(); k++) sorted[k] = items[(size_t)order[k]];

  hg_batch* b = new hg_batch();
  for (size_t k = 0; k < order.size(); k++) {
    const int f = field_of(order[k]);
    if (b->seg_count[f] == 0) b->seg_begin[f] = (int64_t)k;
    b->seg_count[f]++;
  }
  for (int f = 0; f < kNumFields; f++) {
    b->seg_ctas[f] = ctas_for[f];
    b->seg_threads[f] = threads_for[f];
  }
  b->n_problems = n_problems;
  b->n_items = (int64_t)sorted.size();
  b->n_ctas = ctas_for[kGz];
  b->partials = part;
  b->pairs = pairs;
  b->device = device;
  if (n_problems > 0) {
    rc = cuda_check(cudaMalloc(&b->d_probs, sizeof(ProblemDev) * probs.size()), "cudaMalloc");
    if (rc == HG_OK)
      rc = cuda_check(cudaMemcpy(b->d_probs, probs.data(), sizeof(ProblemDev) * probs.size(),
                                 cudaMemcpyHostToDevice),
                      "cudaMemcpy(problems)");
  }
  if (rc == HG_OK && !sorted.empty()) {
    rc = cuda_check(cudaMalloc(&b->d_items, sizeof(WorkItem) * sorted.size()), "cudaMalloc");
    if (rc == HG_OK)
      rc = cuda_check(cudaMemcpy(b->d_items, sorted.data(), sizeof(WorkItem) * sorted.size(),
                                 cudaMemcpyHostToDevice),
                      "cudaMemcpy(items)");
  }
  if (rc != HG_OK) {
    cudaFree(b->d_probs);
    cudaFree(b->d_items);
    delete b;
    return rc;
  }
  *batch = b;
  return HG_OK;
}

int hg_batch_create(const hg_problem* problems, int64_t n_problems, int64_t chunk_prisms,
                    int32_t n_ctas, hg_batch** batch) {
  hg_batch_shape shapes[kNumFields];
  for (int f = 0; f < kNumFields; f++) shapes[f] = hg_batch_shape{chunk_prisms, kThreads, n_ctas};
  return hg_batch_create_shaped(problems, n_problems, shapes, batch);
}

int hg_batch_workspace(const hg_batch* batch, size_t* bytes) {
  if (!batch || !bytes) return set_error(HG_ERR_INVALID, "null pointer");
  *bytes = kCounterBytes + sizeof(double) * (size_t)batch->partials;
  return HG_OK;
}

int hg_batch_info(const hg_batch* batch, int64_t* n_items, int64_t* n_ctas, double* pairs) {
  if (!batch) return set_error(HG_ERR_INVALID, "null batch");
  if (n_items) *n_items = batch->n_items;
  if (n_ctas) *n_ctas = batch->n_ctas;
  if (pairs) *pairs = batch->pairs;
  return HG_OK;
}

int hg_batch_run(const hg_batch* batch, void* workspace, size_t workspace_bytes, void* stream) {
  if (!batch) return set_error(HG_ERR_INVALID, "null batch");
  size_t need = 0;
  hg_batch_workspace(batch, &need);
  if (!workspace || workspace_bytes < need)
    return set_error(HG_ERR_INVALID, "workspace missing or too small");
  if (batch->n_problems == 0) return HG_OK;
  cudaStream_t st = (cudaStream_t)stream;
  unsigned long long* counter = static_cast<unsigned long long*>(workspace);
  double* part = reinterpret_cast<double*>(static_cast<char*>(workspace) + kCounterBytes);
  // one work counter per field
  int rc = cuda_check(cudaMemsetAsync(counter, 0, sizeof(unsigned long long) * kNumFields, st),
                      "cudaMemsetAsync(counter)");
  if (rc != HG_OK) return rc;
  for (int f = 0; f < kNumFields; f++) {
    if (batch->seg_count[f] == 0) continue;
    const int threads = batch->seg_threads[f];
    batch_kernel_for(f, threads)<<<(unsigned)batch->seg_ctas[f], threads, 0, st>>>(
        batch->d_probs, batch->d_items + batch->seg_begin[f], batch->seg_count[f], counter + f,
        part);
    rc = cuda_check(cudaGetLastError(), "batch_kernel launch");
    if (rc != HG_OK) return rc;
    if (f == kPotential) {  // second launch over the same items: the face part
      rc = cuda_check(cudaMemsetAsync(counter + f, 0, sizeof(unsigned long long), st),
                      "cudaMemsetAsync(counter)");
      if (rc != HG_OK) return rc;
      batch_potential_faces_for(threads)<<<(unsigned)batch->seg_ctas[f], threads, 0, st>>>(
          batch->d_probs, batch->d_items + batch->seg_begin[f], batch->seg_count[f],
          counter + f, part);
      rc = cuda_check(cudaGetLastError(), "batch_kernel launch");
      if (rc != HG_OK) return rc;
    }
  }
  dim3 grid(64, (unsigned)batch->n_problems);
  batch_reduce_kernel<<<grid, 256, 0, st>>>(batch->d_probs, part);
  return cuda_check(cudaGetLastError(), "batch_reduce_kernel launch");
}

int hg_batch_destroy(hg_batch* batch) {
  if (!batch) return HG_OK;
  cudaFree(batch->d_probs);
  cudaFree(batch->d_items);
  delete batch;
  return HG_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Rounds for continuous batching: explicit problem table and item list.
namespace hg {
namespace {

template <int F, int PART = 0>
__device__ __forceinline__ void run_plan_item(const hg_problem_plan& P, const hg_work_item& w,
                                              SmemTile& sh, const Tables& T) {
  const int64_t i = (int64_t)w.tile * kThreads + threadIdx.x;
  const bool active = i < P.n_obs;
  const double pe = active ? P.obs_e[i] : 0.0;
  const double pn = active ? P.obs_n[i] : 0.0;
  const double pu = active ? P.obs_u[i] : 0.0;
  const int64_t p0 = (int64_t)w.chunk * P.chunk;
  const int64_t p1 = min(p0 + P.chunk, P.n_prisms);
  double acc[1] = {0.0};
  bool singular = false;
  const bool check = P.check_singular && P.singular_flag != nullptr;
  accumulate<F, ListSource, kTile, PART>(ListSource{P.prisms_soa, P.prism_stride}, p0, p1, pe,
                                         pn, pu, active, check && PART != 2, 1u << F, sh, T,
                                         acc, singular);
  if (singular) atomicOr(P.singular_flag, 1);
  if (active) {
    double* o = P.partials + (int64_t)w.chunk * P.n_obs + i;
    *o = PART == 2 ? *o + acc[0] : acc[0];
  }
}

// Persistent kernel over the work items of one field F in a round (PART:
// run_item(); the potential runs parts 1 and 2 as two launches).
template <int F, int PART = 0>
__global__ void __launch_bounds__(kThreads,
                                  PART == 0 ? BatchMinBlocks<F>::value : HG_FWD_MIN_BLOCKS_PART)
    round_kernel(const hg_problem_plan* __restrict__ probs, const hg_work_item* __restrict__ items,
                 int64_t n_items, unsigned long long* __restrict__ counter) {
  __shared__ SmemTile sh;
  __shared__ SmemTables tabs;
  __shared__ long long next;
  const Tables T = tabs.stage();
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) next = (long long)atomicAdd(counter, 1ull);
    __syncthreads();
    const long long it = next;
    if (it >= n_items) break;
    const hg_work_item w = items[it];
    run_plan_item<F, PART>(probs[w.problem], w, sh, T);
  }
}

using RoundKernel = void (*)(const hg_problem_plan*, const hg_work_item*, int64_t,
                             unsigned long long*);
RoundKernel round_kernel_for(int f) {
  switch (f) {
    case kPotential: return round_kernel<kPotential, 1>;
    case kGe: return round_kernel<kGe>;
    case kGn: return round_kernel<kGn>;
    case kGz: return round_kernel<kGz>;
    case kGee: return round_kernel<kGee>;
    case kGnn: return round_kernel<kGnn>;
    case kGzz: return round_kernel<kGzz>;
    case kGen: return round_kernel<kGen>;
    case kGez: return round_kernel<kGez>;
    default: return round_kernel<kGnz>;
  }
}

__global__ void round_reduce_kernel(const hg_problem_plan* __restrict__ probs,
                                    const int32_t* __restrict__ ids) {
  const hg_problem_plan P = probs[ids[blockIdx.y]];
  const double scale = field_scale(P.field);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < P.n_obs;
       i += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int64_t c = 0; c < P.n_chunks; c++) s += P.partials[c * P.n_obs + i];
    P.out[i] = s * scale;
  }
}

}  // namespace
}  // namespace hg

extern "C" {

int hg_round_run(const hg_problem_plan* problems, const hg_work_item* items,
                 const int64_t* field_counts, int32_t n_ctas, void* counter, void* stream) {
  if (!field_counts || !counter) return set_error(HG_ERR_INVALID, "bad arguments");
  int64_t n_items = 0;
  for (int f = 0; f < kNumFields; f++) {
    if (field_counts[f] < 0) return set_error(HG_ERR_INVALID, "negative item count");
    n_items += field_counts[f];
  }
  if (n_items > 0 && (!problems || !items)) return set_error(HG_ERR_INVALID, "bad arguments");
  cudaStream_t st = (cudaStream_t)stream;
  if (n_items == 0) return HG_OK;
  int sms = kSmCount, device = 0;
  int rc = cuda_check(cudaGetDevice(&device), "cudaGetDevice");
  if (rc != HG_OK) return rc;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  rc = cuda_check(cudaMemsetAsync(counter, 0, sizeof(unsigned long long) * kNumFields, st),
                  "cudaMemsetAsync(counter)");
  if (rc != HG_OK) return rc;
  int64_t begin = 0;
  for (int f = 0; f < kNumFields; f++) {
    const int64_t n = field_counts[f];
    if (n == 0) continue;
    int64_t ctas = n_ctas;
    if (ctas <= 0) {
      int per_sm = 0;
      rc = cuda_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, round_kernel_for(f),
                                                                    kThreads, 0),
                      "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
      if (rc != HG_OK) return rc;
      ctas = (int64_t)std::max(1, per_sm) * sms;
    }
    ctas = std::min<int64_t>(ctas, n);
    unsigned long long* cnt = static_cast<unsigned long long*>(counter) + f;
    round_kernel_for(f)<<<(unsigned)ctas, kThreads, 0, st>>>(problems, items + begin, n, cnt);
    rc = cuda_check(cudaGetLastError(), "round_kernel launch");
    if (rc != HG_OK) return rc;
    if (f == kPotential) {  // second launch over the same items: the face part
      rc = cuda_check(cudaMemsetAsync(cnt, 0, sizeof(unsigned long long), st),
                      "cudaMemsetAsync(counter)");
      if (rc != HG_OK) return rc;
      round_kernel<kPotential, 2><<<(unsigned)ctas, kThreads, 0, st>>>(problems, items + begin, n,
                                                                        cnt);
      rc = cuda_check(cudaGetLastError(), "round_kernel launch");
      if (rc != HG_OK) return rc;
    }
    begin += n;
  }
  return HG_OK;
}

int hg_round_reduce(const hg_problem_plan* problems, const int32_t* problem_ids, int64_t n_ids,
                    void* stream) {
  if (n_ids < 0 || n_ids > 65535 || (n_ids > 0 && (!problems || !problem_ids)))
    return set_error(HG_ERR_INVALID, "bad arguments (at most 65535 problems per reduce)");
  if (n_ids == 0) return HG_OK;
  dim3 grid(64, (unsigned)n_ids);
  round_reduce_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(problems, problem_ids);
  return cuda_check(cudaGetLastError(), "round_reduce_kernel launch");
}

}  // extern "C"
