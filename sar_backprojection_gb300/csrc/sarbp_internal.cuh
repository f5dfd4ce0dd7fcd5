// sarbp_internal.cuh -- shared device-side definitions of the focuser kernels.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/sarbp.h"

namespace sarbp {

// Physical constants of the reference (sar_focuser_puntual_noui.py:24-29):
// speed of light, chirp rate and pi as the float32 literal 3.14159274...
constexpr double kC = 2.9979246e8;
constexpr double kAlfa = 3.335987619777693e11;
constexpr double kPiF32 = 3.141592741012573242;

// Scene constants derived once on the host with the reference's evaluation
// order, passed to every kernel by value.
struct SceneParams {
    int64_t dim0, dim1, npix;
    const double *x, *y, *z;
    const uint8_t *mask;
    const int32_t *index, *sint;
    const double *tx, *ty, *tz;
    const float2 *raw;       // sample (r, a) at raw[a*pitch + r]
    int64_t nra, naz, pitch;
    double near_range, dra, lambda;
    double beta;             // 4*pi*alfa/(c*c)                    (:29)
    double k4pl;             // (-4*pi)/lambda                     (:105)
    double inv_dra;          // 1/dra (reference-range estimate only)
    // float-float / FP32 forms for the mixed path (hi + lo == value to ~2^-48)
    float near_hi, near_lo;  // near range
    float idra_hi, idra_lo;  // 1/dra
    float k1_hi, k1_lo;      // k4pl/(2*pi), turns per metre
    float k2_hi, k2_lo;      // beta/(2*pi), turns per square metre
    float k4pl_f, beta_f, beta2_f, inv_dra_f;
    // the same FP32 values in both halves of a packed f32x2 operand
    unsigned long long inv_dra_f2, beta_f2, magic_f2;
    uint32_t wait_polls;     // staged kernels: polls before a stage wait gives up
    int32_t withhold;        // staged kernels, diagnostic: skip each pass's first copy
};

// Aperture of one pixel, clamped to the kept pulses 0 < a < naz-1
// (sar_focuser_puntual_noui.py:46-55).  Returns false when nothing is kept
// or the pixel is masked (:35-42).
__host__ __device__ inline bool pixel_aperture(uint8_t mask, int32_t sint, int32_t index,
                                               int64_t naz, int64_t *lo, int64_t *hi)
{
    if (mask != 1 || sint == -9999) return false;
    // jj_size = ceil(s/2)*2 + 1 ; offset = ceil(|s|/2), both on integers.
    const int64_t s = sint;
    const int64_t half_up = (s >= 0) ? (s + 1) / 2 : -((-s) / 2);   // ceil(s/2)
    const int64_t jj_size = half_up * 2 + 1;
    const int64_t off = (s >= 0) ? (s + 1) / 2 : ((-s) + 1) / 2;    // ceil(|s|/2)
    if (jj_size <= 0) return false;
    const int64_t a0 = (int64_t)index - off;
    int64_t l = a0 > 1 ? a0 : 1;
    int64_t h = a0 + jj_size - 1;
    if (h > naz - 2) h = naz - 2;
    *lo = l;
    *hi = h;
    return l <= h;
}

// SplitMix64 finaliser of (pulse << 32 | bin): per-pixel checksum term of
// the contributing (pulse, range-bin) pairs.
__host__ __device__ inline uint64_t mix64(int64_t pulse, int64_t bin)
{
    uint64_t z = ((uint64_t)pulse << 32) | (uint64_t)(uint32_t)bin;
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// Exact FP64 range bin of pixel p at pulse a with the reference's rounding
// sequence (no fused multiply-add): sar_focuser_puntual_noui.py:71-95.
// Returns -1 when the bin is outside 0 <= bin < nra-1.
__device__ inline int64_t exact_bin(double px, double py, double pz,
                                    double tx, double ty, double tz,
                                    double near_range, double dra, int64_t nra,
                                    double *r2_out, double *r_out)
{
    const double xc = __dsub_rn(px, tx);
    const double yc = __dsub_rn(py, ty);
    const double zc = __dsub_rn(pz, tz);
    const double r2 = __dadd_rn(__dadd_rn(__dmul_rn(xc, xc), __dmul_rn(yc, yc)),
                                __dmul_rn(zc, zc));
    const double r = __dsqrt_rn(r2);
    const double f = __ddiv_rn(__dsub_rn(r, near_range), dra);
    const double fb = rint(f);
    *r2_out = r2;
    *r_out = r;
    if (!(fb < (double)(nra - 1) && fb >= 0.0)) return -1;
    return (int64_t)fb;
}

// exact_bin with the division by dra replaced by a product with inv_dra =
// RN(1/dra), except near a .5 tie.  With q = (R - near)/dra exactly,
// f = RN((R - near) * inv_dra) is within |q| * 2^-52 of q and the reference's
// RN(q) within |q| * 2^-53, so rint(f) equals the reference's rint(RN(q))
// unless a half-integer lies within |f| * 2^-51 of f; in that band (and only
// there) the correctly rounded quotient is formed.  Same bins, same r2 and r.
__device__ inline int64_t exact_bin_recip(double px, double py, double pz,
                                          double tx, double ty, double tz,
                                          double near_range, double dra, double inv_dra,
                                          int64_t nra, double *r2_out, double *r_out)
{
    const double xc = __dsub_rn(px, tx);
    const double yc = __dsub_rn(py, ty);
    const double zc = __dsub_rn(pz, tz);
    const double r2 = __dadd_rn(__dadd_rn(__dmul_rn(xc, xc), __dmul_rn(yc, yc)),
                                __dmul_rn(zc, zc));
    const double r = __dsqrt_rn(r2);
    const double num = __dsub_rn(r, near_range);
    double f = __dmul_rn(num, inv_dra);
    double fb = rint(f);
    // f - rint(f) is exact; 2^-51 |f| bounds |f - RN(q)| with margin
    if (fabs(__dsub_rn(f, fb)) >= 0.5 - fabs(f) * 0x1p-51 - 0x1p-1000) {
        f = __ddiv_rn(num, dra);
        fb = rint(f);
    }
    *r2_out = r2;
    *r_out = r;
    if (!(fb < (double)(nra - 1) && fb >= 0.0)) return -1;
    return (int64_t)fb;
}

// Device status block at the head of every workspace.
struct StatusBlock {
    unsigned int error;      // non-zero: a bounded wait gave up
    unsigned int where;      // tag of the wait that gave up
    int range[2];            // sarbp_raw_bin_range's reduction (0 between uses)
    unsigned int pad[60];
};

}  // namespace sarbp

// Host-side helpers shared by the translation units (defined in capi.cu).
namespace sarbp {
void set_error(const char *fmt, ...);
bool build_params(const sarbp_scene *s, SceneParams *p);
int cuda_status(cudaError_t e, const char *what);
bool valid_tuning(sarbp_tuning *t);   // fills library defaults, validates
// Clear the thread's error, validate the scene and the tuning (defaults filled).
int mixed_args(const sarbp_scene *scene, const sarbp_tuning *tuning, SceneParams *P,
               sarbp_tuning *T);

// Mixed-path workspace layout (offsets 256-byte aligned).  The first part
// (up to `base`) is the chunk tables every mixed launch needs; staged=2
// adds the cost-ordered tile queue its persistent grid drains (up to
// `total`; total == base otherwise).
struct MixedLayout {
    size_t status;   // StatusBlock
    size_t ptab;     // float4[nchunks*chunk]: e = t(k) - t(k0), |e|^2
    size_t pff;      // PulseFF[naz]: float-float pulse positions
    size_t ctab;     // ChunkRef[nchunks]: bounds of e and t(k0)
    size_t sdev;     // float[nchunks*chunk/32]: chord deviation per 32-pulse stage
    size_t base;     // end of the chunk tables
    int64_t ntiles;  // staged=2: pixel tiles of the scene (0 otherwise)
    size_t keys_in, vals_in, keys_out, vals_out;   // tile costs / ids, sorted
    size_t sort_tmp, sort_tmp_bytes;               // radix-sort scratch
    size_t cursor;   // queue cursor (unsigned long long)
    size_t total;
};
MixedLayout mixed_layout(const SceneParams &P, const sarbp_tuning &T);

int launch_focus_fp64(const SceneParams &P, double *out, int32_t *nvalid, uint64_t *checksum,
                      cudaStream_t stream);
int raw_bin_range(const SceneParams &P, const sarbp_tuning &T, void *workspace, size_t ws_bytes,
                  int64_t *range, cudaStream_t stream);
int raw_bin_range_async(const SceneParams &P, const sarbp_tuning &T, void *workspace,
                        size_t ws_bytes, int32_t *host_range, cudaStream_t stream);
int launch_mixed_range(const SceneParams &P, const sarbp_tuning &T, void *workspace,
                       size_t ws_bytes, int64_t first, int64_t count, double *out,
                       int32_t *nvalid, uint64_t *checksum, uint64_t *counters,
                       cudaStream_t stream);
int tile_queue_keys(const SceneParams &P, const sarbp_tuning &T, void *workspace,
                    size_t ws_bytes, uint32_t *keys, int64_t n, cudaStream_t stream);
int launch_mixed_prepare(const SceneParams &P, const sarbp_tuning &T, void *workspace,
                         size_t ws_bytes, cudaStream_t stream);
int launch_mixed_main(const SceneParams &P, const sarbp_tuning &T, void *workspace,
                      size_t ws_bytes, double *out, int32_t *nvalid, uint64_t *checksum,
                      uint64_t *counters, cudaStream_t stream);

// batches of scenes in one persistent launch (focus_staged.cu)
int64_t batch_workspace_size(int nscenes, int64_t max_items);
int batch_set_scene(void *bws, size_t bytes, int slot, int nscenes, const SceneParams &P,
                    const sarbp_tuning &T, void *scene_ws, size_t scene_ws_bytes, double *out,
                    int32_t *nvalid, uint64_t *checksum, cudaStream_t stream);
int batch_set_items(void *bws, size_t bytes, int nscenes, const int32_t *items, int64_t n,
                    cudaStream_t stream);
int batch_focus(void *bws, size_t bytes, int nscenes, const sarbp_tuning &T, int64_t n_items,
                bool diag, uint64_t *counters, cudaStream_t stream);
int tile_costs(const SceneParams &P, const sarbp_tuning &T, int64_t *costs, cudaStream_t stream);
int tile_order(const SceneParams &P, const sarbp_tuning &T, const MixedLayout &L, char *ws,
               cudaStream_t stream);
size_t tile_sort_bytes(int64_t ntiles);
int tile_count(const SceneParams &P, const sarbp_tuning &T, int64_t *nt);

// host -> device copies (hostcopy.cu): SM loads when the source is mapped
// page-locked host memory (or device memory), the copy engine otherwise
int h2d_bytes(void *dst, const void *src, int64_t bytes, cudaStream_t stream);
// device -> host: SM stores into mapped page-locked memory, else the copy engine
int d2h_bytes(void *dst, const void *src, int64_t bytes, cudaStream_t stream);
int h2d_rows(float2 *dst, int64_t dpitch, const float2 *src, int64_t spitch, int64_t lo,
             int64_t n, int64_t rows, cudaStream_t stream);
// the same rows over the bin interval `bound` holds in memory (no host wait);
// SARBP_EINVAL, nothing enqueued, when the layout does not suit it
int h2d_rows_bound(float2 *dst, int64_t dpitch, const float2 *src, int64_t spitch,
                   const int32_t *bound, int64_t rows, int ctas, cudaStream_t stream);
}  // namespace sarbp
