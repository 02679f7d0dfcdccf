// Compensated FP32 ("double-float") sums for the reductions of the acceleration kernels.
//
// GB300 runs FP64 at a small fraction of its FP32 rate, so the window products of Anderson and
// Broyden and the objective / step-length sums of the trust region, when accumulated in FP64
// element by element, were bound by the FP64 pipe (~85 FP64 operations per vertex for a window of
// 5).  Here a value is an unevaluated sum hi + lo of two floats, carried with error-free
// transformations on the FP32 pipe:
//   * two_sum (Knuth, TAOCP vol. 2, 4.2.2): s + e = a + b exactly;
//   * fast_two_sum (Dekker 1971), for |a| >= |b|;
//   * two_prod with a fused multiply-add: p + e = a * b exactly;
//   * the accurate double-float addition of Hida, Li and Bailey (QD library paper, 2001).
// A sum keeps about 44 significant bits; it is converted to FP64 once per warp.  Every reduction
// order stays fixed, so results remain deterministic.  The operations below use only additions,
// subtractions and explicit fmaf, so contraction by the compiler cannot change them.
#pragma once

#include <cuda_runtime.h>

namespace pbgb {

struct DFloat
{
    float hi, lo;
};

__device__ __forceinline__ DFloat df_two_sum(float a, float b)
{
    float const s  = __fadd_rn(a, b);
    float const bb = __fsub_rn(s, a);
    float const e  = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return {s, e};
}

__device__ __forceinline__ DFloat df_fast_two_sum(float a, float b)
{
    float const s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ DFloat df_two_prod(float a, float b)
{
    float const p = __fmul_rn(a, b);
    return {p, __fmaf_rn(a, b, -p)};
}

__device__ __forceinline__ DFloat df_add(DFloat a, DFloat b)
{
    DFloat s       = df_two_sum(a.hi, b.hi);
    DFloat const t = df_two_sum(a.lo, b.lo);
    s.lo           = __fadd_rn(s.lo, t.hi);
    s              = df_fast_two_sum(s.hi, s.lo);
    s.lo           = __fadd_rn(s.lo, t.lo);
    return df_fast_two_sum(s.hi, s.lo);
}

__device__ __forceinline__ DFloat df_add(DFloat a, float b)
{
    DFloat s = df_two_sum(a.hi, b);
    s.lo     = __fadd_rn(s.lo, a.lo);
    return df_fast_two_sum(s.hi, s.lo);
}

// a . b of two 3-vectors (the w components are ignored), exact products.
__device__ __forceinline__ DFloat df_dot3(float4 a, float4 b)
{
    DFloat s = df_two_prod(a.x, b.x);
    s        = df_add(s, df_two_prod(a.y, b.y));
    return df_add(s, df_two_prod(a.z, b.z));
}

// (a - b)^2 with the difference and the square carried exactly to double-float precision.
__device__ __forceinline__ DFloat df_sq_diff(float a, float b)
{
    DFloat const d = df_two_sum(a, -b);
    DFloat s       = df_two_prod(d.hi, d.hi);
    s.lo           = __fmaf_rn(__fmul_rn(2.f, d.hi), d.lo, s.lo);
    return df_fast_two_sum(s.hi, s.lo);
}

__device__ __forceinline__ DFloat df_shfl_xor(DFloat v, int off)
{
    return {__shfl_xor_sync(0xffffffffu, v.hi, off), __shfl_xor_sync(0xffffffffu, v.lo, off)};
}

// Sum over the warp (butterfly: every lane holds the total).
__device__ __forceinline__ DFloat df_warp_sum(DFloat v)
{
#pragma unroll
    for (int off = 16; off > 0; off >>= 1)
        v = df_add(v, df_shfl_xor(v, off));
    return v;
}

__device__ __forceinline__ double df_to_double(DFloat v)
{
    return double(v.hi) + double(v.lo);
}

} // namespace pbgb
