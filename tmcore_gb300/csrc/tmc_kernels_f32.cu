// FP32 instantiation: FP32 edge/vertex state and stencil arithmetic; FP64
// metrics in memory, FP64 gd and tracer mass, FP64 compensated sums.
#include "tmc_kernels_impl.cuh"

namespace tmc {

TMC_INSTANTIATE(float)

}  // namespace tmc
