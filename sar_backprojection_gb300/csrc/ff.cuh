// ff.cuh -- float-float ("double-single") arithmetic on the FP32 pipe.
//
// GB300 issues FP64 at about 1/75 of its FP32 FMA rate, so the per-(pixel,
// chunk) reference geometry that needs ~1e-11 relative accuracy (slant range
// and phase wrap at kilometre ranges and centimetre wavelength) is computed as
// unevaluated sums hi + lo of two floats.  The error-free transforms are the
// classical ones (Knuth's TwoSum, Dekker's FastTwoSum, TwoProd via FMA); all
// operations use explicitly rounded intrinsics so that no contraction or
// reassociation can break them.
#pragma once

namespace sarbp {

// s + e == a + b exactly, s = fl(a + b).
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e)
{
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// Same, for |a| >= |b|.
__device__ __forceinline__ void fast_two_sum(float a, float b, float &s, float &e)
{
    s = __fadd_rn(a, b);
    e = __fsub_rn(b, __fsub_rn(s, a));
}

// p + e == a * b exactly, p = fl(a * b).
__device__ __forceinline__ void two_prod(float a, float b, float &p, float &e)
{
    p = __fmul_rn(a, b);
    e = __fmaf_rn(a, b, -p);
}

// Nearest integer of x (|x| < 2^22) by the 1.5*2^23 shift, ties to even.
__device__ __forceinline__ float round_shift(float x, int &n)
{
    const float t = __fadd_rn(x, 12582912.0f);
    n = __float_as_int(t) - 0x4B400000;
    return __fsub_rn(t, 12582912.0f);
}

// Difference of two float-float values given as (hi, lo) pairs; the result
// is left unnormalised (|lo| a few ulps of hi at most).
__device__ __forceinline__ void ff_sub(float ah, float al, float bh, float bl, float &sh, float &sl)
{
    two_sum(ah, -bh, sh, sl);
    sl = __fadd_rn(sl, __fsub_rn(al, bl));
}

// (h + l)^2 as hi + lo with the l^2 term kept.
__device__ __forceinline__ void ff_sqr(float h, float l, float &qh, float &ql)
{
    two_prod(h, h, qh, ql);
    ql = __fmaf_rn(__fadd_rn(h, h) + l, l, ql);
}

// sqrt(h + l) as rh + rl, given y ~ 1/sqrt(h) to FP32 accuracy: one Newton
// correction in float-float.
__device__ __forceinline__ void ff_sqrt(float h, float l, float y, float &rh, float &rl)
{
    const float r = __fmul_rn(h, y);
    float q, qe;
    two_prod(r, r, q, qe);
    const float resid = __fadd_rn(__fsub_rn(__fsub_rn(h, q), qe), l);
    const float c = __fmul_rn(resid, __fmul_rn(0.5f, y));
    fast_two_sum(r, c, rh, rl);
}

// (ah + al) * (bh + bl) as ph + pl (al*bl dropped).
__device__ __forceinline__ void ff_mul(float ah, float al, float bh, float bl, float &ph, float &pl)
{
    two_prod(ah, bh, ph, pl);
    pl = __fmaf_rn(ah, bl, __fmaf_rn(al, bh, pl));
}

}  // namespace sarbp
