// staged_c64.cu -- TMA-staged kernels with 64-pulse chunks (one float-float
// reference per 64 pulses), all (tile, window) variants.
#include "staged_kernels.cuh"

namespace sarbp {
SARBP_STAGED_CHUNK_EXTERN(, 64)
}  // namespace sarbp
