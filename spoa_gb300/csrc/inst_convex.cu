// inst_convex.cu - kernels of the convex gap model (compiled on its own so
// the three gap models build in parallel).
#include "poa_kernels.cuh"

namespace spoa_gb300 {
SPOA_GB300_INSTANTIATE(kConvex)
}  // namespace spoa_gb300
