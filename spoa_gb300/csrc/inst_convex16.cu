// inst_convex16.cu - kernels of the convex gap model with 16-bit lanes
// (one translation unit per gap model and width so they build in parallel).
#include "poa_kernels.cuh"

namespace spoa_gb300 {
SPOA_GB300_INSTANTIATE(kConvex, int16_t)
SPOA_GB300_INSTANTIATE_MW(kConvex)
}  // namespace spoa_gb300
