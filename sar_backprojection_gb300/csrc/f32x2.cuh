// f32x2.cuh -- packed FP32 pair arithmetic (Blackwell add/sub/mul/fma.f32x2).
//
// One instruction applies the same IEEE round-to-nearest operation to both
// halves of a 64-bit register pair, so a pair computation gives bit for bit
// the results of the two scalar operations it replaces, in half the issue
// slots.
#pragma once

#include <cstdint>

namespace sarbp {

typedef unsigned long long f2_t;   // (lo, hi) = (first, second) FP32 value

__device__ __forceinline__ f2_t f2_pack(float lo, float hi)
{
    f2_t r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}

__device__ __forceinline__ f2_t f2_dup(float v) { return f2_pack(v, v); }

__device__ __forceinline__ void f2_unpack(f2_t v, float &lo, float &hi)
{
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}

__device__ __forceinline__ f2_t f2_fma(f2_t a, f2_t b, f2_t c)
{
    f2_t d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}

__device__ __forceinline__ f2_t f2_add(f2_t a, f2_t b)
{
    f2_t d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}

__device__ __forceinline__ f2_t f2_sub(f2_t a, f2_t b)
{
    f2_t d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}

__device__ __forceinline__ f2_t f2_mul(f2_t a, f2_t b)
{
    f2_t d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}

// max(a, b, c) in one three-input FP32 max (sm_100 and later).
__device__ __forceinline__ float fmax3(float a, float b, float c)
{
    float d;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}

}  // namespace sarbp
