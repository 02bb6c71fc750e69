// The persistent kernel of the batched forward (prism_batch.cu), shared by
// the translation units that instantiate it for each CTA shape
// (prism_batch.cu: 128 points per CTA, prism_batch64.cu: 64).
#pragma once
#include <cuda_runtime.h>

#include "forward_core.cuh"

namespace hg {

struct ProblemDev {
  const double* e;
  const double* n;
  const double* u;
  int64_t n_obs;
  const double* soa;
  int64_t stride;
  int64_t n_prisms;
  int64_t chunk;        // prisms per work item
  int64_t n_chunks;
  int64_t part_offset;  // first partial (in doubles) of this problem in the workspace
  double* out;
  int32_t* flag;
  int32_t field;
  int32_t check_singular;
};

// One work item: THREADS points (point tile `tile`) x one prism chunk.
struct WorkItem {
  int32_t problem;
  int32_t tile;
  int32_t chunk;
  int32_t pad;
};

// PART (the potential: accumulate()): 0 the whole pairs; 1 writes the
// edge-log part, 2 adds the face part (a second launch over the same items).
template <int F, int THREADS, int PART = 0>
__device__ __forceinline__ void run_item(const ProblemDev& P, const WorkItem& w,
                                         SmemTileT<THREADS>& sh, const Tables& T,
                                         double* __restrict__ part) {
  const int64_t i = (int64_t)w.tile * THREADS + threadIdx.x;
  const bool active = i < P.n_obs;
  const double pe = active ? P.e[i] : 0.0;
  const double pn = active ? P.n[i] : 0.0;
  const double pu = active ? P.u[i] : 0.0;
  const int64_t p0 = (int64_t)w.chunk * P.chunk;
  const int64_t p1 = min(p0 + P.chunk, P.n_prisms);
  double acc[1] = {0.0};
  bool singular = false;
  const bool check = P.check_singular && P.flag != nullptr;
  accumulate<F, ListSource, THREADS, PART>(ListSource{P.soa, P.stride}, p0, p1, pe, pn, pu,
                                           active, check && PART != 2, 1u << F, sh, T, acc,
                                           singular);
  if (singular) atomicOr(P.flag, 1);
  if (active) {
    double* o = part + P.part_offset + (int64_t)w.chunk * P.n_obs + i;
    *o = PART == 2 ? *o + acc[0] : acc[0];
  }
}

// Persistent kernel for the work items of one field F (the items of a batch
// are grouped by field and each group runs its own launch): specialised per
// field, so it keeps that field's register budget and instruction footprint;
// THREADS points per CTA and per work item, THREADS prisms per shared-memory
// tile, and as many resident CTAs per SM as the 128-point kernel times
// 128 / THREADS (the same registers per thread).
template <int F, int THREADS, int PART = 0>
__global__ void __launch_bounds__(THREADS, (PART == 0 ? BatchMinBlocks<F>::value
                                                      : HG_FWD_MIN_BLOCKS_PART) *
                                               (kThreads / THREADS))
    batch_kernel(const ProblemDev* __restrict__ probs, const WorkItem* __restrict__ items,
                 int64_t n_items, unsigned long long* __restrict__ counter,
                 double* __restrict__ part) {
  __shared__ SmemTileT<THREADS> sh;
  __shared__ SmemTables tabs;
  __shared__ long long next;
  const Tables T = tabs.stage();
  for (;;) {
    __syncthreads();  // everyone is done with `next` and the previous tile
    if (threadIdx.x == 0) next = (long long)atomicAdd(counter, 1ull);
    __syncthreads();
    const long long it = next;
    if (it >= n_items) break;
    const WorkItem w = items[it];
    run_item<F, THREADS, PART>(probs[w.problem], w, sh, T, part);
  }
}

using BatchKernel = void (*)(const ProblemDev*, const WorkItem*, int64_t, unsigned long long*,
                             double*);

// The potential runs as two launches over its items (accumulate()): this
// table gives the first (edge-log part), batch_potential_faces the second.
template <int THREADS>
BatchKernel batch_kernel_table(int f) {
  switch (f) {
    case kPotential: return batch_kernel<kPotential, THREADS, 1>;
    case kGe: return batch_kernel<kGe, THREADS>;
    case kGn: return batch_kernel<kGn, THREADS>;
    case kGz: return batch_kernel<kGz, THREADS>;
    case kGee: return batch_kernel<kGee, THREADS>;
    case kGnn: return batch_kernel<kGnn, THREADS>;
    case kGzz: return batch_kernel<kGzz, THREADS>;
    case kGen: return batch_kernel<kGen, THREADS>;
    case kGez: return batch_kernel<kGez, THREADS>;
    default: return batch_kernel<kGnz, THREADS>;
  }
}

template <int THREADS>
BatchKernel batch_potential_faces() {
  return batch_kernel<kPotential, THREADS, 2>;
}

// The kernel of field f for `threads` points per CTA (64 or 128), and the
// potential's second launch; the 64-point kernels are compiled in their own
// translation unit.
BatchKernel batch_kernel_for(int f, int threads);
BatchKernel batch_kernel_for64(int f);
BatchKernel batch_potential_faces_for(int threads);
BatchKernel batch_potential_faces64();

}  // namespace hg
