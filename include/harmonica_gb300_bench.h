/*
 * Benchmark support of harmonica_gb300 (no counterpart in the reference):
 * a probe that measures the FP64 pipe peak of the GPU, the roofline
 * denominator of the FP64-bound prism kernels.
 */
#ifndef HARMONICA_GB300_BENCH_H
#define HARMONICA_GB300_BENCH_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/*
 * Launch n_threads_total threads (a multiple of 256) that each run
 * 16 * iters FP64 flops (independent fused multiply-adds) and write one
 * double to out[n_threads_total] (device memory).  Asynchronous on `stream`.
 * Returns 0 (HG_OK), or HG_ERR_INVALID (-1) on bad arguments / HG_ERR_CUDA (-2)
 * on a launch failure, with the message in hg_last_error().
 */
int hg_fp64_peak_probe(double *out, int64_t n_threads_total, int iters, void *stream);

#ifdef __cplusplus
}
#endif

#endif
