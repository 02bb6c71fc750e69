// The 64-point-per-CTA kernels of the batched forward (batch_core.cuh), in
// their own translation unit so that the two CTA shapes compile in parallel.
#include "batch_core.cuh"

namespace hg {

BatchKernel batch_kernel_for64(int f) { return batch_kernel_table<64>(f); }
BatchKernel batch_potential_faces64() { return batch_potential_faces<64>(); }

}  // namespace hg
