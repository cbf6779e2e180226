// sl_vdw_energy.cuh -- the exact form's write-step van der Waals potential of
// a pair out of contact (ColliderSingleCore.cpp:228-240), with the far pairs
// evaluated on the FP32 pipe.
//
// The reference's closed form, U = -Ha/6 (2RaRb/S + 2RaRb/T + ln(S/T)) with
// S = z^2 - (Ra + Rb)^2, T = z^2 - (Ra - Rb)^2, z = Ra + Rb + h, costs two
// FP64 divisions, a third inside the logarithm, and the logarithm itself --
// about three times a pair's force on GB300's narrow FP64 pipe.  With
// D = z^2 - Ra^2 - Rb^2 = S + 2RaRb and w = 2RaRb / D, S = D (1 - w) and
// T = D (1 + w), and the bracket is
//     2w / (1 - w^2) - 2 atanh(w) = sum_{j >= 1} 4j/(2j+1) w^(2j+1),
// a series of positive terms (no cancellation, where the closed form
// cancels from O(w) to O(w^3)).  For w <= 1/4 (z >= 1.58 radius sums for
// equal radii: all but the nearest neighbours) thirteen terms leave a
// truncation of about 3e-16 relative; they are summed by Horner in
// double-float arithmetic (sl_df.cuh, ~46 bits) on the FP32 pipe, so a pair
// costs about ten FP64 operations instead of ~70.  Nearer pairs take the
// closed form.  The energy totals are compared with the reference's to
// 1e-10 relative (the GPU sums the pairs in another order anyway); a far
// pair's value here is within ~1e-13 of the exact bracket, closer than the
// reference's own cancelling closed form.
#pragma once
#include "sl_device.cuh"
#include "sl_df.cuh"
#include "sl_pair_exact.cuh"

namespace sl {

namespace vdwdf {

// x as hi + lo: hi = RN_f32(x), lo = RN_f32(x - hi) (the difference is exact
// in FP64).  For the positive, normal-range lengths and areas used here.
__device__ __forceinline__ df::F2 from_double(double x)
{
    const float hi = d2f_bits(x, 0);
    return {hi, d2f_bits(x - f2d_bits(hi), 0)};
}

__device__ __forceinline__ df::F2 mul(df::F2 a, df::F2 b)
{
    df::F2 p = df::two_prod(a.hi, b.hi);
    p.lo = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, p.lo));
    return df::fast_two_sum(p.hi, p.lo);
}

// a / b for b > 0: q1 = a.hi / b.hi, then one correction from the remainder
// a - q1 b formed with an exact product.
__device__ __forceinline__ df::F2 div(df::F2 a, df::F2 b)
{
    const float q1 = a.hi / b.hi;
    const df::F2 p = df::two_prod(q1, b.hi);
    const float r = (((a.hi - p.hi) - p.lo) + a.lo) - q1 * b.lo;
    return df::fast_two_sum(q1, r / b.hi);
}

// 4j / (2j + 1) as hi + lo, j = 1..13
struct Coef {
    float hi, lo;
};
__host__ __device__ constexpr Coef coef(int j)
{
    return Coef{(float)(4.0 * j / (2.0 * j + 1.0)),
                (float)(4.0 * j / (2.0 * j + 1.0) - (double)(float)(4.0 * j / (2.0 * j + 1.0)))};
}

}  // namespace vdwdf

// U_vdw of a pair out of contact with gap h >= h_min (the value the
// reference adds to PE at ColliderSingleCore.cpp:239).
__device__ __forceinline__ double vdw_energy_far_df(double Ha, double h, double Ra, double Rb, double twoRa)
{
    const double sum = Ra + Rb;
    const double S = h * (h + (sum + sum));  // z^2 - (Ra + Rb)^2
    const double two_RaRb = twoRa * Rb;
    if (!(3.0 * two_RaRb <= S)) return vdw_energy(Ha, h, Ra, Rb, twoRa);  // w > 1/4: the closed form
    using namespace vdwdf;
    const df::F2 w = div(from_double(two_RaRb), from_double(S + two_RaRb));
    const df::F2 x = df::sqr(w);
    constexpr Coef c13 = coef(13);
    df::F2 p{c13.hi, c13.lo};
#pragma unroll
    for (int j = 12; j >= 1; --j) {
        const Coef c = coef(j);
        p = df::add(mul(p, x), df::F2{c.hi, c.lo});
    }
    const df::F2 bracket = mul(mul(w, x), p);  // sum_j 4j/(2j+1) w^(2j+1)
    return -Ha / 6 * (f2d_bits(bracket.hi) + f2d_bits(bracket.lo));
}

}  // namespace sl
