// FP64 pipe peak probe used by bench.py for the roofline denominator: every
// thread runs 8 independent fused multiply-add chains, so the launch is bound
// by the FP64 pipe alone.  Each thread executes 16 * iters FP64 flops
// (8 chains x iters FMAs x 2 flops).
#include <cuda_runtime.h>

#include <string>

#include "../../include/harmonica_gb300.h"
#include "../../include/harmonica_gb300_bench.h"

namespace hg {
int set_error(int code, const std::string& msg);
int cuda_check(cudaError_t e, const char* what);
}  // namespace hg

namespace {

__global__ void fp64_fma_chains(double* out, int iters, double a, double b) {
  double x0 = threadIdx.x * 1e-3, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
  double x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; i++) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

}  // namespace

extern "C" int hg_fp64_peak_probe(double* out, int64_t n_threads_total, int iters, void* stream) {
  const int threads = 256;
  if (!out) return hg::set_error(HG_ERR_INVALID, "null pointer");
  if (n_threads_total <= 0 || n_threads_total % threads != 0 || iters <= 0)
    return hg::set_error(HG_ERR_INVALID, "bad arguments (threads: a positive multiple of 256)");
  fp64_fma_chains<<<(unsigned)(n_threads_total / threads), threads, 0, (cudaStream_t)stream>>>(
      out, iters, 0.999999, 1e-6);
  return hg::cuda_check(cudaGetLastError(), "fp64 peak probe launch");
}
