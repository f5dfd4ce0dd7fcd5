// staged_c128.cu -- TMA-staged kernels with 128-pulse chunks (one float-float
// reference per 128 pulses), all (tile, window) variants.
#include "staged_kernels.cuh"

namespace sarbp {
SARBP_STAGED_CHUNK_EXTERN(, 128)
}  // namespace sarbp
