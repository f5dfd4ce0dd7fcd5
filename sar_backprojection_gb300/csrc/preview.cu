// preview.cu -- 8-bit amplitude preview of a focused image.
//
// The reference's visualiser (img_visualizer.py:23-46) shows |image| scaled
// so that 15 x the mean amplitude maps to 255:
//   normalized = clip(|x| * (255 / (15 * mean|x|)), 0, 255).astype(uint8)
// Here: one pass of fixed-order partial sums of |x| (a fixed grid, one
// partial per block, so the mean is the same on every run), then a pass in
// which every block sums the partials in the same order, forms the scale
// and writes the bytes.  |x| is hypot(re, im) in FP64, the product by the
// scale is FP64, the cast truncates (NumPy's astype), NaN gives 0.
#include <algorithm>

#include "sarbp_internal.cuh"

namespace sarbp {

constexpr int kPreviewThreads = 256;

__device__ __forceinline__ double block_sum(double v, double *red)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) red[w] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) s += red[k];
    __syncthreads();
    return s;   // valid in thread 0
}

__global__ void __launch_bounds__(kPreviewThreads)
amplitude_partial_kernel(const double2 *__restrict__ img, int64_t npix,
                         double *__restrict__ partials)
{
    __shared__ double red[kPreviewThreads / 32];
    double acc = 0.0;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < npix; i += stride) {
        const double2 v = img[i];
        acc += hypot(v.x, v.y);
    }
    const double s = block_sum(acc, red);
    if (threadIdx.x == 0) partials[blockIdx.x] = s;
}

__global__ void __launch_bounds__(kPreviewThreads)
amplitude_u8_kernel(const double2 *__restrict__ img, int64_t npix,
                    const double *__restrict__ partials, int nparts, double scale_factor,
                    uint8_t *__restrict__ out, double *__restrict__ mean_out)
{
    __shared__ double red[kPreviewThreads / 32];
    __shared__ double s_scale;
    double acc = 0.0;
    for (int k = threadIdx.x; k < nparts; k += blockDim.x) acc += partials[k];
    const double total = block_sum(acc, red);
    if (threadIdx.x == 0) {
        const double mean = total / (double)npix;
        const double max_val = scale_factor * mean;
        s_scale = 255.0 / max_val;
        if (blockIdx.x == 0 && mean_out) *mean_out = mean;
    }
    __syncthreads();
    const double c = s_scale;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < npix; i += stride) {
        const double2 v = img[i];
        const double x = hypot(v.x, v.y) * c;
        // clip to [0, 255], then truncate; NaN (0 * inf) gives 0
        const double y = x >= 0.0 ? fmin(x, 255.0) : 0.0;
        out[i] = (uint8_t)(int)y;
    }
}

}  // namespace sarbp

using namespace sarbp;

extern "C" SARBP_API int sarbp_amplitude_u8(const double *image, int64_t npix,
                                            double scale_factor, uint8_t *out, double *mean,
                                            double *scratch, size_t scratch_bytes, void *stream)
{
    if (!image || !out || !scratch || npix <= 0 || !(scale_factor > 0.0)) {
        set_error("sarbp_amplitude_u8: bad pointers, pixel count or scale factor");
        return SARBP_EINVAL;
    }
    int dev = 0, sms = 0;
    int rc = cuda_status(cudaGetDevice(&dev), "sarbp_amplitude_u8: device");
    if (rc) return rc;
    rc = cuda_status(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev),
                     "sarbp_amplitude_u8: SM count");
    if (rc) return rc;
    // a grid of whole waves (8 blocks of 256 threads per SM), capped by the
    // scratch (one partial per block) and by the pixels
    int64_t grid = (int64_t)sms * 8;
    grid = std::min<int64_t>(grid, (int64_t)(scratch_bytes / sizeof(double)));
    grid = std::min<int64_t>(grid, (npix + kPreviewThreads - 1) / kPreviewThreads);
    if (grid < 1) {
        set_error("sarbp_amplitude_u8: scratch of %zu bytes holds no partial sum", scratch_bytes);
        return SARBP_EWORKSPACE;
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const double2 *img = reinterpret_cast<const double2 *>(image);
    amplitude_partial_kernel<<<(unsigned)grid, kPreviewThreads, 0, s>>>(img, npix, scratch);
    rc = cuda_status(cudaGetLastError(), "amplitude_partial launch");
    if (rc) return rc;
    amplitude_u8_kernel<<<(unsigned)grid, kPreviewThreads, 0, s>>>(img, npix, scratch, (int)grid,
                                                                  scale_factor, out, mean);
    return cuda_status(cudaGetLastError(), "amplitude_u8 launch");
}
