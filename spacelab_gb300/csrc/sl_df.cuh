// sl_df.cuh -- double-float arithmetic: a value held as an unevaluated sum
// hi + lo of two FP32 numbers (|lo| <= ulp(hi)/2), about 48 significant
// bits, built from error-free transformations on the FP32 pipe (Knuth's
// TwoSum, Dekker's Fast2Sum, and the FMA-based TwoProduct).  The mixed form
// uses it where it needs more than FP32: pair displacements, |r|^2, the
// squared gap and the per-sphere sums.  GB300's FP32 pipe is ~72x its FP64
// pipe, so these few FP32 operations cost far less than one FP64 operation.
//
// Every function here must be compiled without reassociation of FP32
// additions (nvcc's default); the FMAs are explicit.
#pragma once
#include <cuda_runtime.h>

namespace sl {
namespace df {

struct F2 {
    float hi, lo;
};

// s + e == a + b exactly (any a, b without overflow)
__device__ __forceinline__ F2 two_sum(float a, float b)
{
    const float s = a + b;
    const float bp = s - a;
    const float e = (a - (s - bp)) + (b - bp);
    return {s, e};
}

// s + e == a + b exactly when |a| >= |b| (or a == 0)
__device__ __forceinline__ F2 fast_two_sum(float a, float b)
{
    const float s = a + b;
    return {s, b - (s - a)};
}

// p + e == a * b exactly (barring underflow)
__device__ __forceinline__ F2 two_prod(float a, float b)
{
    const float p = a * b;
    return {p, fmaf(a, b, -p)};
}

__device__ __forceinline__ F2 add(F2 a, F2 b)
{
    F2 s = two_sum(a.hi, b.hi);
    s.lo += a.lo + b.lo;
    return fast_two_sum(s.hi, s.lo);
}

__device__ __forceinline__ F2 sub(F2 a, F2 b)
{
    F2 s = two_sum(a.hi, -b.hi);
    s.lo += a.lo - b.lo;
    return fast_two_sum(s.hi, s.lo);
}

__device__ __forceinline__ F2 sqr(F2 a)
{
    F2 p = two_prod(a.hi, a.hi);
    p.lo = fmaf(2.0f * a.hi, a.lo, p.lo);
    return fast_two_sum(p.hi, p.lo);
}

// Compensated running sum (Neumaier): s carries the sum, c the exact
// rounding errors of each addition; the value is s + c.
struct Sum {
    float s, c;
    __device__ __forceinline__ void add(float v)
    {
        const F2 t = two_sum(s, v);
        s = t.hi;
        c += t.lo;
    }
};

}  // namespace df
}  // namespace sl
