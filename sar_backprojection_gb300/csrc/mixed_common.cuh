// mixed_common.cuh -- per-pixel-chunk setup and per-pulse body shared by the
// mixed-precision kernels.
//
// Precision plan (per pixel p, per pulse chunk with reference pulse k0):
//   FP64, once per (pixel, chunk): d0 = p - t(k0), R0 = |d0|, the reference
//     range bin n0 = rint((R0 - near)/dra) with FP32 remainder g0, and the
//     reference phase phi0 = (-4*pi/lambda)*R0 + beta*R0^2 wrapped to turns.
//   FP32, per pulse k: e = t(k) - t(k0) (from a per-pulse table),
//     D  = R(k)^2 - R0^2 = -2 d0.e + |e|^2                     (3 FFMA)
//     dR = R(k) - R0 = R0*(sqrt(1+u)-1), u = D/R0^2, as the series
//          D*(c1 + D*(c2 + D*c3))                                (3 ops)
//     bin = n0 + rint(g0 + dR/dra), re-derived in FP64 when the FP32 value
//          lies within kAmbiguity of a .5 tie, so bins equal the FP64 path's
//     dphi = dR*(a + beta*dR), a = -4*pi/lambda + 2*beta*R0
//     term = R(k)^2 * raw(bin, k) * exp(-j*dphi), summed in FP32 per chunk
//   per chunk: rotate the chunk sum by exp(-j*phi0) and add it to a
//     Kahan-compensated FP32 accumulator.
// When the chunk's differential range is too large for the FP32 series
// (|u| bound > kUMax) the chunk is processed with the exact FP64 body.
#pragma once

#include "sarbp_internal.cuh"

namespace sarbp {

// |fr| above this (fr = g - rint(g) in [-0.5, 0.5]) re-derives the bin in FP64.
// The FP32 error of g is below ~2e-6 bins for |u| <= kUMax (see DESIGN).
constexpr float kAmbiguity = 0.5f - 3.0517578125e-05f;   // 0.5 - 2^-15
constexpr float kUMax = 4.0e-3f;      // series validity bound on |D|/R0^2
constexpr float kDRMax = 16.0f;       // metres; keeps |dphi| small in FP32
constexpr double kInv2Pi = 0.15915494309189533577;

// Per-chunk bound of |e| components (x, y, z) and of |e|^2 (w).
// Per-pulse entry: e = t(k) - t(k0) (x, y, z) and |e|^2 (w), FP32.
struct ChunkSetup {
    float mx, my, mz;     // -2*d0
    float c1, c2, c3;     // series coefficients of dR(D)
    float g0;             // FP32 remainder of the reference bin position
    float a;              // -4*pi/lambda + 2*beta*R0 (rad/m)
    float r0sq;           // R0^2
    float w0re, w0im;     // exp(-j*phi0)
    int n0;               // reference range bin
    bool exact;           // chunk needs the FP64 body
};

// FP64 setup of one (pixel, chunk).
__device__ __forceinline__ void chunk_setup(const SceneParams &P, double px, double py, double pz,
                                            int64_t k0, float4 emax, ChunkSetup &S)
{
    const double dx = px - __ldg(P.tx + k0);
    const double dy = py - __ldg(P.ty + k0);
    const double dz = pz - __ldg(P.tz + k0);
    const double r0sq = fma(dx, dx, fma(dy, dy, dz * dz));
    // 1/R0 from the FP32 reciprocal square root plus one FP64 Newton step
    // (relative error ~1e-14), then R0 = R0^2/R0.
    double rs = (double)rsqrtf((float)r0sq);
    rs = rs * fma(-0.5 * r0sq, rs * rs, 1.5);
    const double r0 = r0sq * rs;
    const double f0 = (r0 - P.near_range) * P.inv_dra;
    const double n0d = rint(f0);
    const double ph0 = r0 * fma(P.beta, r0, P.k4pl);
    const double turns = ph0 * kInv2Pi;
    const float frac = (float)(turns - rint(turns));
    float s0, c0;
    sincospif(2.0f * frac, &s0, &c0);
    const float irs = (float)rs;
    S.mx = (float)(-2.0 * dx);
    S.my = (float)(-2.0 * dy);
    S.mz = (float)(-2.0 * dz);
    S.c1 = 0.5f * irs;
    const float ir2 = irs * irs;
    S.c2 = -0.125f * ir2 * irs;
    S.c3 = 0.0625f * ir2 * ir2 * irs;
    S.g0 = (float)(f0 - n0d);
    S.a = (float)fma(2.0 * P.beta, r0, P.k4pl);
    S.r0sq = (float)r0sq;
    S.w0re = c0;
    S.w0im = -s0;
    // Conservative |D| bound over the chunk and the resulting |u|, |dR|.
    const float dmax = fabsf(S.mx) * emax.x + fabsf(S.my) * emax.y + fabsf(S.mz) * emax.z + emax.w;
    const float umax = dmax * ir2;
    const bool bin_ok = fabs(n0d) < 1.0e9;
    S.n0 = bin_ok ? (int)n0d : 0;
    S.exact = !(umax <= kUMax) || !(dmax * S.c1 <= kDRMax) || !bin_ok;
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
__device__ __noinline__ bool exact_term(const SceneParams &P, double px, double py, double pz,
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
