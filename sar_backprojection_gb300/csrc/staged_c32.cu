// staged_c32.cu -- TMA-staged kernels with 32-pulse chunks (one float-float
// reference per 32 pulses), all (tile, window) variants.
#include "staged_kernels.cuh"

namespace sarbp {
SARBP_STAGED_CHUNK_EXTERN(, 32)
}  // namespace sarbp
