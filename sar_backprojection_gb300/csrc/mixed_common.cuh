// mixed_common.cuh -- per-pixel-chunk setup and tie resolution shared by the
// mixed-precision kernels.
//
// Precision plan (per pixel p, per pulse chunk with reference pulse k0):
//   float-float (~44-bit), once per (pixel, chunk): d0 = p - t(k0),
//     R0 = |d0|, the reference bin position f0 = (R0 - near)/dra split into
//     the integer n0 and the FP32 remainder g0, and the reference phase in
//     turns, phi0/2pi = R0*(k4pl + beta*R0)/2pi, wrapped to [-1/2, 1/2].
//   FP32, per pulse k: e = t(k) - t(k0) (per-pulse table),
//     D  = R(k)^2 - R0^2 = -2 d0.e + |e|^2                     (3 FFMA)
//     dR = R(k) - R0 = R0*(sqrt(1+u)-1), u = D/R0^2, as the series
//          D*(c1 + D*(c2 + D*c3))                                (3 ops)
//     bin = n0 + rint(g0 + dR/dra); when the FP32 value lies within the
//          chunk's error bound of a .5 tie it is re-derived (float-float
//          first, FP64 with the reference's exact operation sequence only
//          within 1e-8 bin of the tie), so bins equal the FP64 path's
//     dphi = dR*(a + beta*dR), a = -4*pi/lambda + 2*beta*R0
//     term = R(k)^2 * raw(bin, k) * exp(-j*dphi), summed in FP32 per chunk
//   per chunk: rotate the chunk sum by exp(-j*phi0) and add it to a
//     Kahan-compensated FP32 accumulator.
// When the chunk's differential range is too large for the FP32 series
// (|u| bound > kUMax) the chunk is processed with the exact FP64 body.
// No FP64 instruction runs on the common path (GB300's FP64 pipe issues at
// about 1/75 of its FP32 FMA rate).
#pragma once

#include "ff.cuh"
#include "sarbp_internal.cuh"

namespace sarbp {

constexpr float kUMax = 4.0e-3f;      // series validity bound on |D|/R0^2
constexpr float kDRMax = 16.0f;       // metres; keeps |dphi| small in FP32
// Tie band: |fr| > 0.5 - eps, eps = kEpsRel*|dR|max/dra + kEpsAbs, where
// 6e-7*|dR|max/dra + 1e-6 bounds the FP32 error of g: the roundings of the
// FP32 products -2*d0.e and |e|^2 (relative 2^-24 of terms up to |D|), the
// three FMAs of D, the series (its truncation < 4e-8 m at |u| <= 4e-3) and
// the FP32 1/dra, each a relative error of a few 2^-24 of dR/dra, plus the
// float-float reference g0 (< 1e-9 bin).
constexpr float kEpsRel = 1.5e-6f;
constexpr float kEpsAbs = 2.0e-6f;

// Per-chunk reference record (chunk table).
struct ChunkRef {
    float4 emax;   // max |e_x|, |e_y|, |e_z| and max |e|^2 over the chunk
    float4 thi;    // t(k0) as float-float: hi parts (x, y, z, -)
    float4 tlo;    //                       lo parts
};

// Per-pulse float-float positions, read only when a tie is re-derived.
struct PulseFF {
    float4 hi;
    float4 lo;
};

struct ChunkSetup {
    float mx, my, mz;     // -2*d0
    float c1, c2, c3;     // series coefficients of dR(D)
    float g0;             // FP32 remainder of the reference bin position
    float a;              // -4*pi/lambda + 2*beta*R0 (rad/m)
    float r0sq;           // R0^2
    float w0re, w0im;     // exp(-j*phi0)
    float eps;            // tie band half-width (bins)
    int n0;               // reference range bin
    bool exact;           // chunk needs the FP64 body
};

// Pixel position as float-float, from the FP64 DEM (once per pixel).
struct PixelFF {
    float xh, xl, yh, yl, zh, zl;
};

__device__ __forceinline__ void split_ff(double d, float &h, float &l)
{
    h = __double2float_rn(d);
    l = __double2float_rn(d - (double)h);
}

__device__ __forceinline__ PixelFF pixel_ff(double x, double y, double z)
{
    PixelFF p;
    split_ff(x, p.xh, p.xl);
    split_ff(y, p.yh, p.yl);
    split_ff(z, p.zh, p.zl);
    return p;
}

// |p - t|^2 as float-float (qh + ql); also returns d = p - t rounded to FP32
// (hi + lo of the float-float difference: the hi part alone ignores the lo
// parts of both positions, ~1e-3 m at 20 km coordinates).
__device__ __forceinline__ void ff_dist2(const PixelFF &p, float4 th, float4 tl, float &qh,
                                         float &ql, float &dx, float &dy, float &dz)
{
    float xh, xl, yh, yl, zh, zl;
    ff_sub(p.xh, p.xl, th.x, tl.x, xh, xl);
    ff_sub(p.yh, p.yl, th.y, tl.y, yh, yl);
    ff_sub(p.zh, p.zl, th.z, tl.z, zh, zl);
    dx = __fadd_rn(xh, xl);
    dy = __fadd_rn(yh, yl);
    dz = __fadd_rn(zh, zl);
    float ax, axl, ay, ayl, az, azl;
    ff_sqr(xh, xl, ax, axl);
    ff_sqr(yh, yl, ay, ayl);
    ff_sqr(zh, zl, az, azl);
    float s1, e1, s2, e2;
    two_sum(ax, ay, s1, e1);
    two_sum(s1, az, s2, e2);
    const float l = __fadd_rn(__fadd_rn(__fadd_rn(e1, e2), __fadd_rn(axl, ayl)), azl);
    fast_two_sum(s2, l, qh, ql);
}

// Float-float setup of one (pixel, chunk).
__device__ __forceinline__ void chunk_setup(const SceneParams &P, const PixelFF &p,
                                            const ChunkRef &ref, ChunkSetup &S)
{
    float qh, ql, dx, dy, dz;
    ff_dist2(p, ref.thi, ref.tlo, qh, ql, dx, dy, dz);
    float y = rsqrtf(qh);
    y = __fmul_rn(y, __fmaf_rn(-0.5f * qh, __fmul_rn(y, y), 1.5f));
    float rh, rl;
    ff_sqrt(qh, ql, y, rh, rl);
    // f0 = (R0 - near) * (1/dra)
    float ah, al;
    ff_sub(rh, rl, P.near_hi, P.near_lo, ah, al);
    float fh, fl;
    ff_mul(ah, al, P.idra_hi, P.idra_lo, fh, fl);
    int n0;
    const float fr0 = round_shift(fh, n0);
    S.g0 = __fadd_rn(__fsub_rn(fh, fr0), fl);
    S.n0 = n0;
    // phi0 in turns: R0*(K1 + K2*R0), K1 = k4pl/2pi, K2 = beta/2pi
    float kh, kl;
    ff_mul(P.k2_hi, P.k2_lo, rh, rl, kh, kl);
    float bh, bl;
    two_sum(P.k1_hi, kh, bh, bl);
    bl = __fadd_rn(bl, __fadd_rn(P.k1_lo, kl));
    float th, tl;
    ff_mul(bh, bl, rh, rl, th, tl);
    int nt;
    const float tr = round_shift(th, nt);
    const float frac = __fadd_rn(__fsub_rn(th, tr), tl);
    float s0, c0;
    __sincosf(6.28318530717958648f * frac, &s0, &c0);
    S.w0re = c0;
    S.w0im = -s0;
    S.mx = -2.0f * dx;
    S.my = -2.0f * dy;
    S.mz = -2.0f * dz;
    S.c1 = 0.5f * y;
    const float y2 = y * y;
    S.c2 = -0.125f * y2 * y;
    S.c3 = 0.0625f * y2 * y2 * y;
    S.a = fmaf(P.beta2_f, rh, P.k4pl_f);
    S.r0sq = qh;
    // Conservative |D| bound over the chunk and the resulting |u|, |dR|.
    const float4 em = ref.emax;
    const float dmax = fabsf(S.mx) * em.x + fabsf(S.my) * em.y + fabsf(S.mz) * em.z + em.w;
    const float drmax = dmax * S.c1;
    S.eps = fmaf(kEpsRel, drmax * P.inv_dra_f, kEpsAbs);
    S.exact = !(dmax * y2 <= kUMax) || !(drmax <= kDRMax) || !(fabsf(fh) < 4.0e6f) ||
              !(fabsf(th) < 4.0e6f);
}

// Range bin of pixel ii (float-float position p) at pulse a for an ambiguous
// FP32 estimate: float-float first (|error| < ~2e-10 bin); the reference's
// exact FP64 operation sequence (on the FP64 DEM and trajectory) only when
// the float-float value is within 1e-8 bin (plus 2e-11 relative) of the tie.
// Returns -1 when the bin is outside 0 <= bin < nra-1.
static __device__ __noinline__ int resolve_bin(const SceneParams &P, const PixelFF &p, int64_t ii,
                                        const PulseFF *__restrict__ pff, int64_t a)
{
    const float4 th = __ldg(&pff[a].hi), tl = __ldg(&pff[a].lo);
    float qh, ql, dx, dy, dz;
    ff_dist2(p, th, tl, qh, ql, dx, dy, dz);
    float y = rsqrtf(qh);
    y = __fmul_rn(y, __fmaf_rn(-0.5f * qh, __fmul_rn(y, y), 1.5f));
    float rh, rl;
    ff_sqrt(qh, ql, y, rh, rl);
    float ah, al;
    ff_sub(rh, rl, P.near_hi, P.near_lo, ah, al);
    float fh, fl;
    ff_mul(ah, al, P.idra_hi, P.idra_lo, fh, fl);
    int n;
    const float d = __fsub_rn(fh, round_shift(fh, n));      // exact, |d| <= 0.5
    // |d + fl| - 0.5, evaluated without rounding d + fl near 0.5
    const float dist = __fadd_rn(__fsub_rn(fabsf(d), 0.5f), d >= 0.f ? fl : -fl);
    if (fabsf(dist) > fmaf(2.0e-11f, fabsf(fh), 1.0e-8f)) {
        int bin = n;
        if (dist > 0.f) bin = d >= 0.f ? n + 1 : n - 1;
        return (bin >= 0 && (int64_t)bin < P.nra - 1) ? bin : -1;
    }
    double r2, r;
    return (int)exact_bin(__ldg(P.x + ii), __ldg(P.y + ii), __ldg(P.z + ii), __ldg(P.tx + a),
                          __ldg(P.ty + a), __ldg(P.tz + a), P.near_range, P.dra, P.nra, &r2, &r);
}

// Kahan-compensated add of x into (s, c).
__device__ __forceinline__ void kahan_add(float &s, float &c, float x)
{
    const float y = __fsub_rn(x, c);
    const float t = __fadd_rn(s, y);
    c = __fsub_rn(__fsub_rn(t, s), y);
    s = t;
}

// Exact FP64 contribution of pulse a (the FP64 kernel's body) with its
// absolute phase: R^2 * raw * exp(-j*phi).  Returns false if not kept.
static __device__ __noinline__ bool exact_term(const SceneParams &P, double px, double py, double pz,
                                        int64_t a, int64_t *bin_out, double *tre, double *tim)
{
    double r2, r;
    const int64_t bin = exact_bin(px, py, pz, __ldg(P.tx + a), __ldg(P.ty + a), __ldg(P.tz + a),
                                  P.near_range, P.dra, P.nra, &r2, &r);
    *bin_out = bin;
    if (bin < 0) return false;
    const double phase = __dadd_rn(__dmul_rn(P.k4pl, r), __dmul_rn(P.beta, r2));
    double fs, fc;
    sincos(-phase, &fs, &fc);
    const float2 v = __ldg(P.raw + a * P.pitch + bin);
    const double A = r2 * (double)v.x, B = r2 * (double)v.y;
    *tre = A * fc - B * fs;
    *tim = A * fs + B * fc;
    return true;
}

}  // namespace sarbp
