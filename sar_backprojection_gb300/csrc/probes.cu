// probes.cu -- issue-rate probes: the roofline denominators of this workload.
//
// The focuser is bound by instruction issue (FP32 FMA lanes, the SFU that
// evaluates sin/cos, FP64 on the plain kernel), not by HBM or tensor cores,
// so its roofline needs the device's FP32-FMA, SFU and FP64-FMA throughput.
// Each probe runs enough independent dependency chains per thread to saturate
// its pipe, on a grid of 8 CTAs x 256 threads per SM, and is timed with CUDA
// events on the caller's stream.
#include "sarbp_internal.cuh"

namespace sarbp {

constexpr int kProbeIters = 4096;

__device__ double g_probe_sink[256];

__global__ void __launch_bounds__(256) probe_ffma(float *sink, float seed)
{
    float a0 = seed + threadIdx.x, a1 = a0 + 1.f, a2 = a0 + 2.f, a3 = a0 + 3.f;
    float a4 = a0 + 4.f, a5 = a0 + 5.f, a6 = a0 + 6.f, a7 = a0 + 7.f;
    const float m = 0.999999f, c = 1e-7f;
#pragma unroll 16
    for (int i = 0; i < kProbeIters; ++i) {
        a0 = fmaf(a0, m, c); a1 = fmaf(a1, m, c); a2 = fmaf(a2, m, c); a3 = fmaf(a3, m, c);
        a4 = fmaf(a4, m, c); a5 = fmaf(a5, m, c); a6 = fmaf(a6, m, c); a7 = fmaf(a7, m, c);
    }
    const float s = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
    if (s == 1.2345f) sink[threadIdx.x] = s;
}

__global__ void __launch_bounds__(256) probe_mufu(float *sink, float seed)
{
    float a0 = seed + threadIdx.x * 1e-3f, a1 = a0 + 0.1f, a2 = a0 + 0.2f, a3 = a0 + 0.3f;
#pragma unroll 16
    for (int i = 0; i < kProbeIters; ++i) {
        a0 = __sinf(a0); a1 = __sinf(a1); a2 = __sinf(a2); a3 = __sinf(a3);
    }
    const float s = a0 + a1 + a2 + a3;
    if (s == 1.2345f) sink[threadIdx.x] = s;
}

__global__ void __launch_bounds__(256) probe_dfma(double *sink, double seed)
{
    double a0 = seed + threadIdx.x, a1 = a0 + 1.0, a2 = a0 + 2.0, a3 = a0 + 3.0;
    const double m = 0.999999999, c = 1e-9;
#pragma unroll 8
    for (int i = 0; i < kProbeIters / 16; ++i) {
        a0 = fma(a0, m, c); a1 = fma(a1, m, c); a2 = fma(a2, m, c); a3 = fma(a3, m, c);
    }
    const double s = a0 + a1 + a2 + a3;
    if (s == 1.2345) sink[threadIdx.x] = s;
}

}  // namespace sarbp

using namespace sarbp;

extern "C" SARBP_API int sarbp_probe_issue_rates(double *rates, void *stream_ptr)
{
    if (!rates) {
        set_error("sarbp_probe_issue_rates: rates is NULL");
        return SARBP_EINVAL;
    }
    cudaStream_t stream = static_cast<cudaStream_t>(stream_ptr);
    int dev = 0, sms = 0;
    int rc = cuda_status(cudaGetDevice(&dev), "cudaGetDevice");
    if (rc) return rc;
    rc = cuda_status(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev),
                     "cudaDeviceGetAttribute");
    if (rc) return rc;
    void *sinkp = nullptr;
    rc = cuda_status(cudaGetSymbolAddress(&sinkp, g_probe_sink), "cudaGetSymbolAddress");
    if (rc) return rc;
    const unsigned blocks = (unsigned)sms * 8u;
    const double threads = (double)blocks * 256.0;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float ms = 0.f;
    // warm-up of each probe, then a timed run
    for (int which = 0; which < 3; ++which) {
        for (int rep = 0; rep < 2; ++rep) {
            if (rep == 1) cudaEventRecord(e0, stream);
            if (which == 0)
                probe_ffma<<<blocks, 256, 0, stream>>>((float *)sinkp, 1.0f);
            else if (which == 1)
                probe_mufu<<<blocks, 256, 0, stream>>>((float *)sinkp, 0.5f);
            else
                probe_dfma<<<blocks, 256, 0, stream>>>((double *)sinkp, 1.0);
            if (rep == 1) cudaEventRecord(e1, stream);
        }
        rc = cuda_status(cudaEventSynchronize(e1), "probe");
        if (rc) break;
        cudaEventElapsedTime(&ms, e0, e1);
        const double ops = which == 0 ? threads * kProbeIters * 8.0
                         : which == 1 ? threads * kProbeIters * 4.0
                                      : threads * (kProbeIters / 16) * 4.0;
        rates[which] = ops / (ms * 1e-3);
    }
    rates[3] = (double)sms;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return rc;
}
