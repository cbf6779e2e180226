// sl_fp64_exact.cuh -- correctly rounded FP64 quotients and square roots
// with most of the work on the integer pipe.
//
// GB300's FP64 pipe runs at ~1/72 of its FP32 rate, and an IEEE double
// division or square root costs ~7.5 FP64 slots.  Here each of them costs
// one FP64 multiply (an estimate within a few units in the last place) and
// an exact rounding decision made with integer arithmetic:
//   quotient  q0 ~ a/b.  With a = ma 2^ea, b = mb 2^eb, q0 = mq 2^eq (53-bit
//             integer significands), the exact remainder
//             D = ma 2^s - mb mq  (s = ea - eb - eq, 106-bit products)
//             measures a/b - q0 = D / mb in units of q0's last place; the
//             correctly rounded significand is mq + k, k = the integer
//             nearest D/mb, found by comparing 2D with odd multiples of mb.
//   sqrt      s0 ~ sqrt(x).  With x = mx 2^ex, s0 = ms 2^es, sqrt(x) lies
//             above the midpoint ms + j + 1/2 iff 4 mx 2^t > (2ms + 2j + 1)^2
//             (t = ex - 2 es), all 108-bit integers; no ties are possible.
// Any case outside the fast path -- zero, subnormal, Inf/NaN operands, an
// estimate more than 4 units off, or a result that would leave the
// estimate's binade -- falls back to the hardware operation, so the result
// is always the IEEE round-to-nearest-even value.  Tested bit for bit
// against the hardware operations in tests/test_gpu_parity.py.
#pragma once
#include <cstdint>
#include <cstring>
#include <cuda_runtime.h>

#include "sl_device.cuh"

namespace sl {

namespace fx {

// The hardware operations of the (rare) fallbacks, kept out of line so that
// the inlined fast paths stay compact.
static __device__ __noinline__ double hw_div(double a, double b) { return a / b; }
static __device__ __noinline__ double hw_sqrt(double x) { return sqrt(x); }

constexpr unsigned long long kMant = 0xfffffffffffffull;
constexpr unsigned long long kHidden = 1ull << 52;

// 128-bit helpers (hi, lo as unsigned 64-bit words)
__device__ __forceinline__ void mul128(unsigned long long a, unsigned long long b, unsigned long long& hi,
                                       unsigned long long& lo)
{
    lo = a * b;
    hi = __umul64hi(a, b);
}

// x = (hi, lo) as a signed 128-bit number known to fit in 64 bits -> ok
__device__ __forceinline__ bool fits64(unsigned long long hi, unsigned long long lo)
{
    return (hi == 0ull && (long long)lo >= 0) || (hi == ~0ull && (long long)lo < 0);
}

}  // namespace fx

// RN(a / b) from an estimate mq * 2^(eq - 1075) of a / b (mq nominally in
// [2^52, 2^53)), or its negation -RN(a / b) = RN(-a / b) when NEG.  The
// rounding decision uses the exact remainder D = ma 2^s - mb mq, which
// measures a / b - mq in units of mq's last place as D / mb.
//   FULL = true   checks all 128 bits of D and accepts corrections k of
//                 -1..2, so any estimate is safe (a poor one only takes the
//                 fallback); the estimates here are within (-1, 2.1) units.
//   FULL = false  keeps the low 64 bits of D and is valid only for a LOWER
//                 estimate within 1.5 units (0 <= D < 1.5 mb): k is 0 or 1.
template <bool FULL, bool NEG = false>
__device__ __forceinline__ double div_round(double a, double b, unsigned long long mq, int eq)
{
    using namespace fx;
    const unsigned long long ba = (unsigned long long)__double_as_longlong(a);
    const unsigned long long bb = (unsigned long long)__double_as_longlong(b);
    const int ea = (int)((ba >> 52) & 0x7ff), eb = (int)((bb >> 52) & 0x7ff);
    const unsigned long long sgn = ((ba ^ bb) & 0x8000000000000000ull) ^ (NEG ? 0x8000000000000000ull : 0ull);
    const int s = ea - eb - eq + 1075;
    bool ok = ea != 0 && ea != 0x7ff && eb != 0 && eb != 0x7ff && eq >= 1 && eq <= 2046 && (s == 52 || s == 53);
    const int sh = s == 53 ? 53 : 52;
    const unsigned long long ma = (ba & kMant) | kHidden, mb = (bb & kMant) | kHidden;
    const unsigned long long llo = ma << sh, plo = mb * mq;
    const long long D = (long long)(llo - plo);
    const long long D2 = 2 * D;
    const long long m = (long long)mb, m3 = 3 * m;
    int k;
    if (FULL) {
        const unsigned long long lhi = ma >> (64 - sh), phi = __umul64hi(mb, mq);
        ok &= fits64(lhi - phi - (llo < plo ? 1ull : 0ull), llo - plo);
        ok &= (D < (1ll << 60)) & (D > -(1ll << 60));
        // k = nearest integer to D/mb in -1..2 (branch-free); ties
        // D2 == odd * mb cannot occur for a quotient of 53-bit numbers but
        // are sent to the fallback all the same
        k = (int)(D2 > m) + (int)(D2 > m3) - (int)(D2 < -m);
        ok &= (D2 > -m3) & (D2 < 5 * m) & (D2 != m) & (D2 != -m) & (D2 != m3);
    } else {
        k = (int)(D2 > m);
        ok &= (D2 >= 0) & (D2 < m3) & (D2 != m);
    }
    const unsigned long long mr = mq + (long long)k;
    ok &= mr >= kHidden && mr < (kHidden << 1);
    const unsigned long long res = sgn | ((unsigned long long)eq << 52) | (mr & kMant);
    if (__builtin_expect(!ok, 0)) return NEG ? -hw_div(a, b) : hw_div(a, b);
    return __longlong_as_double((long long)res);
}

// RN(a / b) given q0, an estimate of a / b within a few units in its last
// place (typically RN(a * y) for y ~ 1/b).
__device__ __forceinline__ double div_from_estimate(double a, double b, double q0)
{
    const unsigned long long bq = (unsigned long long)__double_as_longlong(q0);
    const unsigned long long ba = (unsigned long long)__double_as_longlong(a);
    const unsigned long long bb = (unsigned long long)__double_as_longlong(b);
    const int eq = (int)((bq >> 52) & 0x7ff);
    // a wrong-signed estimate is pushed out of range so that it falls back
    const bool sign_ok = ((bq ^ ba ^ bb) & 0x8000000000000000ull) == 0;
    return div_round<true>(a, b, (bq & fx::kMant) | fx::kHidden, sign_ok && eq != 0x7ff ? eq : 0);
}

// RN(sqrt(x)) from an estimate ms * 2^(es - 1075) (ms nominally in
// [2^52, 2^53)); x > 0.  All 128 bits of the comparison are checked and
// corrections of -1..2 units are accepted, so any estimate is safe (a poor
// one only takes the fallback).
__device__ __forceinline__ double sqrt_round(double x, unsigned long long ms, int es)
{
    using namespace fx;
    const unsigned long long bx = (unsigned long long)__double_as_longlong(x);
    const int ex = (int)((bx >> 52) & 0x7ff);
    const int t = ex - 2 * es + 1075;  // x = mx 2^(ex-1075), estimate = ms 2^(es-1075)
    bool ok = ex != 0 && ex != 0x7ff && (bx >> 63) == 0 && es >= 1 && es <= 2046 && (t == 52 || t == 53) &&
              ms < (kHidden << 1);
    const unsigned long long mx = (bx & kMant) | kHidden;
    // X4 = mx 2^(t+2): compare with C_j = (2 ms + j)^2 for odd j
    const int sh = t == 53 ? 55 : 54;
    const unsigned long long xhi = mx >> (64 - sh), xlo = mx << sh;
    const unsigned long long two = 2 * ms;  // < 2^54
    unsigned long long chi, clo;
    mul128(two, two, chi, clo);            // (2ms)^2
    // X4 - (2ms)^2 as signed; |.| < 2^62 on the fast path
    const unsigned long long dlo = xlo - clo;
    const unsigned long long dhi = xhi - chi - (xlo < clo ? 1ull : 0ull);
    ok &= fits64(dhi, dlo);
    const long long E = (long long)dlo;   // X4 - 4 ms^2
    // C_j - 4 ms^2 = 4 ms j + j^2
    const long long f = (long long)(2 * two);  // 4 ms  (< 2^55)
    // sqrt(x) is above ms + j/2 (odd j) iff E > j f + j^2; k in -1..2 (the
    // estimates here are within (-1, 2) units)
    const int k = (int)(E > f + 1) + (int)(E > 3 * f + 9) - (int)(E < -f + 1);
    ok &= (E < 5 * f + 25) & (E > -3 * f + 9);
    const unsigned long long mr = ms + (long long)k;
    ok &= mr >= kHidden && mr < (kHidden << 1);
    const unsigned long long res = ((unsigned long long)es << 52) | (mr & kMant);
    if (__builtin_expect(!ok, 0)) return hw_sqrt(x);
    return __longlong_as_double((long long)res);
}

// RN(sqrt(x)) given s0, an estimate of sqrt(x) within a few units in its
// last place; x > 0.
__device__ __forceinline__ double sqrt_from_estimate(double x, double s0)
{
    const unsigned long long bs = (unsigned long long)__double_as_longlong(s0);
    const int es = (int)((bs >> 52) & 0x7ff);
    const bool good = (bs >> 63) == 0 && es != 0 && es != 0x7ff;
    return sqrt_round(x, (bs & fx::kMant) | fx::kHidden, good ? es : 0);
}

// y / 2 for a normal y by decrementing the exponent (integer pipe)
__device__ __forceinline__ double half_of(double y)
{
    return __longlong_as_double(__double_as_longlong(y) - (1ll << 52));
}

// 1/sqrt(x) to within ~1 unit in the last place for x in the FP32 normal
// range: an FP32 seed (conversions on the integer pipe) and two Newton steps
// y <- y + (y/2)(1 - x y^2), 6 FP64 operations.  Outside that range the
// result is not normal and the callers fall back to the hardware operations.
__device__ __forceinline__ double rsqrt_refined(double x)
{
    const double y0 = f2d_bits(rsqrtf(d2f_bits(x, 0)));
    const double t0 = x * y0;
    const double e0 = fma(-t0, y0, 1.0);
    const double y1 = fma(half_of(y0), e0, y0);
    const double t1 = x * y1;
    const double e1 = fma(-t1, y1, 1.0);
    return fma(half_of(y1), e1, y1);
}

// ---------------------------------------------------------------------------
// Estimates on the integer pipe.  A reciprocal significand is held as a
// 64-bit fixed-point number R ~ 2^116 / mb (mb = the divisor's 53-bit
// significand), so R is in (2^63, 2^64).  The quotient estimate of a / b is
// then the high half of (ma 2^11) * R, with no FP64 operation.

// floor((2^116 - 1) / mb) for mb in [2^52, 2^53): restoring division of the
// all-ones numerator, one quotient bit per step (set-up code only).
__host__ __device__ inline unsigned long long recip_sig(unsigned long long mb)
{
    unsigned long long q = 0, rem = 0;
    for (int bit = 115; bit >= 0; --bit) {
        rem = (rem << 1) | 1ull;  // rem < mb < 2^53 before the shift
        if (rem >= mb) {
            rem -= mb;
            if (bit < 64) q |= 1ull << bit;
        }
    }
    return q;
}

__host__ __device__ inline unsigned long long recip_of(double b)
{
    unsigned long long bits;
    memcpy(&bits, &b, sizeof bits);
    return recip_sig((bits & fx::kMant) | fx::kHidden);
}

namespace fx {

// 2 u as a 64-bit fixed-point value, saturating at 2^64 - 1
__device__ __forceinline__ unsigned long long twice_sat(unsigned long long u)
{
    return (u >> 63) ? ~0ull : (u << 1);
}

// 2^64 * r for a float r in about [0.25, 1]: its 24-bit significand placed
// by its exponent, saturating at 2^64 - 1
__device__ __forceinline__ unsigned long long float_to_fix64(float r)
{
    const unsigned rb = __float_as_uint(r);
    const int sh = (int)(rb >> 23) - 86;  // 2^64 r = m24 2^(e - 150 + 64)
    const unsigned long long m = (rb & 0x7fffffu) | 0x800000u;
    return sh >= 41 ? ~0ull : (sh < 0 ? 0ull : m << sh);
}

}  // namespace fx

// R ~ 2^116 / mb for the significand mb of b, to about 2^-60: a 24-bit
// seed (rcp.approx.ftz.f32 of the top significand bits) and two Newton
// steps r <- r (2 - g r) in 64-bit fixed point, g = mb / 2^52 in [1, 2).
__device__ __forceinline__ unsigned long long recip_newton(double b)
{
    using namespace fx;
    const unsigned long long bb = (unsigned long long)__double_as_longlong(b);
    const unsigned long long mb = (bb & kMant) | kHidden;
    const float g = __uint_as_float(0x3f800000u | (unsigned)((mb >> 29) & 0x7fffffu));
    float r0;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r0) : "f"(g));
    unsigned long long R = float_to_fix64(r0);
    const unsigned long long G = mb << 11;  // g 2^63
#pragma unroll
    for (int it = 0; it < 2; ++it) {
        const unsigned long long T = __umul64hi(G, R);  // g r 2^63
        R = twice_sat(__umul64hi(R, 0ull - T));         // r (2 - g r) 2^64
    }
    return R;
}

// div_round<false, NEG> out of line: the near-midpoint quotients of
// div_by_fixed, about 3 in 1024.
template <bool NEG>
__device__ __noinline__ double div_near_mid(double a, double b, unsigned long long mq, int eq)
{
    return div_round<false, NEG>(a, b, mq, eq);
}

// RN(a / b) (or -RN(a / b) when NEG) given R ~ 2^116 / mb.
//   FULL = true   for R from recip_newton: the estimate goes through
//                 div_round's 128-bit remainder check.
//   FULL = false  for R from recip_sig.  Then H = floor(ma 2^11 R / 2^64)
//                 lies below T = (ma / mb) 2^63 by less than 2.0001 units
//                 (R is below 2^116 / mb by less than 1 + 2^-52, ma 2^11 <
//                 2^64, and each truncation only lowers the value).  The
//                 low bits L of H that the significand drops decide the
//                 rounding directly unless T's fraction can straddle the
//                 midpoint, i.e. L is within 2 units below it (about 3 in
//                 1024 quotients); those take the exact remainder test.
//                 A quotient of 53-bit numbers is never a midpoint.
template <bool FULL, bool NEG = false>
__device__ __forceinline__ double div_by_fixed(double a, double b, unsigned long long R)
{
    using namespace fx;
    const unsigned long long ba = (unsigned long long)__double_as_longlong(a);
    const unsigned long long bb = (unsigned long long)__double_as_longlong(b);
    const int ea = (int)((ba >> 52) & 0x7ff), eb = (int)((bb >> 52) & 0x7ff);
    const unsigned long long ma = (ba & kMant) | kHidden;
    const unsigned long long H = __umul64hi(ma << 11, R);  // (ma / mb) 2^63, in (2^62, 2^64)
    const int c = (int)(H >> 63);
    const unsigned long long mq = H >> (10 + c);
    const int eq = ea - eb + 1022 + c;
    if (FULL) return div_round<true, NEG>(a, b, mq, eq);
    const unsigned L = (unsigned)H & ((2u << (9 + c)) - 1u);  // dropped bits
    const unsigned half = 1u << (9 + c);
    if (__builtin_expect(L + 2u >= half && L <= half, 0)) return div_near_mid<NEG>(a, b, mq, eq);
    const unsigned long long mr = mq + (L > half ? 1ull : 0ull);
    const bool ok = ea != 0 && ea != 0x7ff && eb != 0 && eb != 0x7ff && eq >= 1 && eq <= 2045 && mr >= kHidden;
    const unsigned long long sgn = ((ba ^ bb) & 0x8000000000000000ull) ^ (NEG ? 0x8000000000000000ull : 0ull);
    // mr == 2^53 carries into the exponent field, which is the right result
    const unsigned long long res = sgn | (((unsigned long long)eq << 52) + (mr - kHidden));
    if (__builtin_expect(!ok, 0)) return NEG ? -fx::hw_div(a, b) : fx::hw_div(a, b);
    return __longlong_as_double((long long)res);
}

// 1/sqrt(x) for a positive normal x = f 2^(2p), f in [1, 4): returns
// Y ~ 2^64 / sqrt(f) (to about 2^-60; Y in (2^63, 2^64)) and sets p and
// F = f 2^62.  A 24-bit seed (rsqrt.approx.ftz.f32 of f's top bits) and two
// Newton steps y <- y (3 - f y^2) / 2 in 64-bit fixed point.  For other x the
// outputs are meaningless and the users below fall back.
__device__ __forceinline__ unsigned long long rsqrt_fix(double x, int& p, unsigned long long& F)
{
    using namespace fx;
    const unsigned long long bx = (unsigned long long)__double_as_longlong(x);
    const int E = (int)((bx >> 52) & 0x7ff) - 1023;
    const int odd = E & 1;
    p = (E - odd) >> 1;
    const unsigned long long mx = (bx & kMant) | kHidden;
    F = mx << (10 + odd);
    const float f = __uint_as_float(((127u + (unsigned)odd) << 23) | (unsigned)((mx >> 29) & 0x7fffffu));
    float y0;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y0) : "f"(f));
    unsigned long long Y = float_to_fix64(y0);
#pragma unroll
    for (int it = 0; it < 2; ++it) {
        const unsigned long long S = __umul64hi(Y, Y);     // y^2 2^64
        const unsigned long long T = __umul64hi(S, F);     // f y^2 2^62
        Y = twice_sat(__umul64hi(Y, (3ull << 62) - T));    // y (3 - f y^2) 2^63 -> y' 2^64
    }
    return Y;
}

// RN(sqrt(x)) from rsqrt_fix(x): sqrt(f) 2^62 = F Y / 2^64.
__device__ __forceinline__ double sqrt_fix(double x, unsigned long long F, unsigned long long Y, int p)
{
    return sqrt_round(x, __umul64hi(F, Y) >> 10, p + 1023);
}

// RN(a / d) for d = RN(sqrt(x)), from rsqrt_fix(x) = (Y, p).
__device__ __forceinline__ double div_by_rsqrt(double a, double d, unsigned long long Y, int p)
{
    using namespace fx;
    const unsigned long long ba = (unsigned long long)__double_as_longlong(a);
    const int ea = (int)((ba >> 52) & 0x7ff);
    const unsigned long long ma = (ba & kMant) | kHidden;
    const unsigned long long H = __umul64hi(ma << 11, Y);  // (ma / sqrt f) 2^11, in (2^62, 2^64)
    const int c = (int)(H >> 63);
    return div_round<true>(a, d, H >> (10 + c), ea - p - 1 + c);
}

// RN(a * b) on the integer pipe: the 106-bit product of the significands
// from one 64x64 high product H = floor(ma mb 2^22 / 2^64) and the low 64
// bits Lo, which together hold it exactly; the bits H drops below the
// 53-bit significand (L) and Lo != 0 (sticky) decide round-to-nearest-even.
// Zero, subnormal, Inf/NaN operands and results outside the normal range
// take the hardware multiply.
__device__ __forceinline__ double mul_int(double a, double b)
{
    using namespace fx;
    const unsigned long long ba = (unsigned long long)__double_as_longlong(a);
    const unsigned long long bb = (unsigned long long)__double_as_longlong(b);
    const int ea = (int)((ba >> 52) & 0x7ff), eb = (int)((bb >> 52) & 0x7ff);
    const unsigned long long x = ((ba & kMant) | kHidden) << 11, y = ((bb & kMant) | kHidden) << 11;
    const unsigned long long H = __umul64hi(x, y);  // in [2^62, 2^64)
    const unsigned long long Lo = x * y;
    const int c = (int)(H >> 63);
    const unsigned long long mq = H >> (10 + c);
    const unsigned L = (unsigned)H & ((2u << (9 + c)) - 1u);
    const unsigned half = 1u << (9 + c);
    const bool up = L > half || (L == half && (Lo != 0ull || (mq & 1ull)));
    const int e = ea + eb - 1023 + c;
    const bool ok = ea != 0 && ea != 0x7ff && eb != 0 && eb != 0x7ff && e >= 1 && e <= 2045;
    const unsigned long long sgn = (ba ^ bb) & 0x8000000000000000ull;
    // mq + up == 2^53 carries into the exponent field, which is the right result
    const unsigned long long res = sgn | (((unsigned long long)e << 52) + (mq + (up ? 1ull : 0ull) - kHidden));
    if (__builtin_expect(!ok, 0)) return a * b;
    return __longlong_as_double((long long)res);
}

}  // namespace sl
