// inst_affine.cu - kernels of the affine gap model (compiled on its own so
// the three gap models build in parallel).
#include "poa_kernels.cuh"

namespace spoa_gb300 {
SPOA_GB300_INSTANTIATE(kAffine)
}  // namespace spoa_gb300
