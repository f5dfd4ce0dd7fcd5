// focus_fp64.cu -- plain FP64 back-projection: one thread per output pixel.
//
// The straightforward GPU form of the reference's per-pixel focusing
// (sar_focuser_puntual_noui.py:9-144) with the CPU path's semantics, which the
// reference's own CuPy kernel (gpu_small_dataset.py:9-108) does not keep:
// round-half-to-even range bins, bins kept iff 0 <= bin < Nra-1, pulses kept
// iff 0 < a < Naz-1.  Every geometry operation is an explicitly rounded IEEE
// op (no FMA contraction) so that range bins are bit-identical to the FP64
// CPU result; the division by DeltaRange is a product with its reciprocal
// except within a tie band where only the correctly rounded quotient decides
// the bin (exact_bin_recip); cos/sin are CUDA's double-precision functions.
//
// Raw data are read where they lie in HBM, in the reference's column-major
// (Nra, Naz) complex64 layout: no host-side transpose into split planes.
// This kernel is the FP64 comparator for the mixed-precision path.
#include <cstdio>

#include "sarbp_internal.cuh"

namespace sarbp {

template <bool kChecksum>
__global__ void __launch_bounds__(128)
focus_fp64_kernel(const SceneParams P, double2 *__restrict__ out,
                  int32_t *__restrict__ nvalid, uint64_t *__restrict__ checksum)
{
    const int64_t ii = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (ii >= P.npix) return;

    double sum_re = 0.0, sum_im = 0.0;
    int64_t n = 0;
    uint64_t cs = 0;
    int64_t lo, hi;
    if (pixel_aperture(P.mask[ii], P.sint[ii], P.index[ii], P.naz, &lo, &hi)) {
        const double px = P.x[ii], py = P.y[ii], pz = P.z[ii];
        const double inv_dra = __ddiv_rn(1.0, P.dra);
        for (int64_t a = lo; a <= hi; ++a) {
            double r2, r;
            const int64_t bin = exact_bin_recip(px, py, pz, __ldg(P.tx + a), __ldg(P.ty + a),
                                                __ldg(P.tz + a), P.near_range, P.dra, inv_dra,
                                                P.nra, &r2, &r);
            if (bin < 0) continue;
            // phase = ((-4*pi)/lambda)*R + beta*R^2 ; filter = exp(-j*phase)
            const double phase = __dadd_rn(__dmul_rn(P.k4pl, r), __dmul_rn(P.beta, r2));
            double fs, fc;
            sincos(-phase, &fs, &fc);
            const float2 v = __ldg(P.raw + a * P.pitch + bin);
            const double A = __dmul_rn(r2, (double)v.x);
            const double B = __dmul_rn(r2, (double)v.y);
            sum_re = __dadd_rn(sum_re, __dsub_rn(__dmul_rn(A, fc), __dmul_rn(B, fs)));
            sum_im = __dadd_rn(sum_im, __dadd_rn(__dmul_rn(A, fs), __dmul_rn(B, fc)));
            ++n;
            if (kChecksum) cs += mix64(a, bin);
        }
    }
    double2 res = make_double2(0.0, 0.0);
    if (n > 0) {
        const double inv = __ddiv_rn(1.0, (double)n);
        res = make_double2(__dmul_rn(sum_re, inv), __dmul_rn(sum_im, inv));
    }
    out[ii] = res;
    if (nvalid) nvalid[ii] = (int32_t)n;
    if (kChecksum) checksum[ii] = cs;
}

int launch_focus_fp64(const SceneParams &P, double *out, int32_t *nvalid, uint64_t *checksum,
                      cudaStream_t stream)
{
    const int threads = 128;
    const int64_t blocks = (P.npix + threads - 1) / threads;
    if (blocks > 0x7fffffffLL) {
        set_error("sarbp_focus_fp64: %lld pixels exceed the launch limit", (long long)P.npix);
        return SARBP_ERANGE;
    }
    if (checksum)
        focus_fp64_kernel<true><<<(unsigned)blocks, threads, 0, stream>>>(
            P, reinterpret_cast<double2 *>(out), nvalid, checksum);
    else
        focus_fp64_kernel<false><<<(unsigned)blocks, threads, 0, stream>>>(
            P, reinterpret_cast<double2 *>(out), nvalid, nullptr);
    return cuda_status(cudaGetLastError(), "focus_fp64 launch");
}

}  // namespace sarbp
