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
#include <cuda_runtime.h>

#include "sl_device.cuh"

namespace sl {

namespace fx {

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

// RN(a / b) given q0, an estimate of a / b within a few units in its last
// place (typically RN(a * y) for y ~ 1/b).
__device__ __forceinline__ double div_from_estimate(double a, double b, double q0)
{
    using namespace fx;
    const unsigned long long ba = (unsigned long long)__double_as_longlong(a);
    const unsigned long long bb = (unsigned long long)__double_as_longlong(b);
    const unsigned long long bq = (unsigned long long)__double_as_longlong(q0);
    const int ea = (int)((ba >> 52) & 0x7ff), eb = (int)((bb >> 52) & 0x7ff), eq = (int)((bq >> 52) & 0x7ff);
    const unsigned long long sgn = (ba ^ bb) & 0x8000000000000000ull;
    const int s = ea - eb - eq + 1075;
    bool ok = ea != 0 && ea != 0x7ff && eb != 0 && eb != 0x7ff && eq != 0 && eq != 0x7ff &&
              ((bq & 0x8000000000000000ull) == sgn) && (s == 52 || s == 53);
    unsigned long long res = 0;
    if (ok) {
        const unsigned long long ma = (ba & kMant) | kHidden, mb = (bb & kMant) | kHidden, mq = (bq & kMant) | kHidden;
        unsigned long long phi, plo;
        mul128(mb, mq, phi, plo);
        const unsigned long long lhi = ma >> (64 - s), llo = ma << s;
        const unsigned long long dlo = llo - plo;
        const unsigned long long dhi = lhi - phi - (llo < plo ? 1ull : 0ull);
        ok = fits64(dhi, dlo);
        const long long D2 = 2 * (long long)dlo;  // |D| < 2^55 on the fast path
        const long long m = (long long)mb, m3 = 3 * m, m5 = 5 * m, m7 = 7 * m, m9 = 9 * m;
        // k = nearest integer to D/mb, |k| <= 4, as a sum of comparisons
        // (branch-free); ties D2 == odd * mb cannot occur for a quotient of
        // 53-bit numbers but are sent to the fallback all the same
        const int k = (int)(D2 > m) + (int)(D2 > m3) + (int)(D2 > m5) + (int)(D2 > m7) - (int)(D2 < -m) -
                      (int)(D2 < -m3) - (int)(D2 < -m5) - (int)(D2 < -m7);
        ok &= (D2 < m9) & (D2 > -m9) & (D2 != m) & (D2 != -m) & (D2 != m3) & (D2 != -m3) & (D2 != m5) &
              (D2 != -m5) & (D2 != m7) & (D2 != -m7);
        const unsigned long long mr = mq + (long long)k;
        ok &= mr >= kHidden && mr < (kHidden << 1);
        res = sgn | ((unsigned long long)eq << 52) | (mr & kMant);
    }
    if (__builtin_expect(!ok, 0)) return a / b;
    return __longlong_as_double((long long)res);
}

// RN(sqrt(x)) given s0, an estimate of sqrt(x) within a few units in its
// last place; x > 0.
__device__ __forceinline__ double sqrt_from_estimate(double x, double s0)
{
    using namespace fx;
    const unsigned long long bx = (unsigned long long)__double_as_longlong(x);
    const unsigned long long bs = (unsigned long long)__double_as_longlong(s0);
    const int ex = (int)((bx >> 52) & 0x7ff), es = (int)((bs >> 52) & 0x7ff);
    const int t = ex - 2 * es + 1075;  // x = mx 2^(ex-1075), s0 = ms 2^(es-1075)
    bool ok = ex != 0 && ex != 0x7ff && es != 0 && es != 0x7ff && (bx >> 63) == 0 && (bs >> 63) == 0 &&
              (t == 52 || t == 53);
    unsigned long long res = 0;
    if (ok) {
        const unsigned long long mx = (bx & kMant) | kHidden, ms = (bs & kMant) | kHidden;
        // X4 = mx 2^(t+2): compare with C_j = (2 ms + j)^2 for odd j
        const int sh = t + 2;  // 54 or 55
        const unsigned long long xhi = mx >> (64 - sh), xlo = mx << sh;
        const unsigned long long two = 2 * ms;  // < 2^54
        unsigned long long chi, clo;
        mul128(two, two, chi, clo);            // (2ms)^2
        // X4 - (2ms)^2 as signed; |.| < 2^62 on the fast path
        const unsigned long long dlo = xlo - clo;
        const unsigned long long dhi = xhi - chi - (xlo < clo ? 1ull : 0ull);
        ok = fits64(dhi, dlo);
        const long long E = (long long)dlo;   // X4 - 4 ms^2
        // C_j - 4 ms^2 = 4 ms j + j^2
        const long long f = (long long)(2 * two);  // 4 ms  (< 2^55)
        // sqrt(x) is above ms + j/2 (odd j) iff E > j f + j^2; |k| <= 4
        const int k = (int)(E > f + 1) + (int)(E > 3 * f + 9) + (int)(E > 5 * f + 25) + (int)(E > 7 * f + 49) -
                      (int)(E < -f + 1) - (int)(E < -3 * f + 9) - (int)(E < -5 * f + 25) - (int)(E < -7 * f + 49);
        ok &= (E < 9 * f + 81) & (E > -9 * f + 81);
        const unsigned long long mr = ms + (long long)k;
        ok &= mr >= kHidden && mr < (kHidden << 1);
        res = ((unsigned long long)es << 52) | (mr & kMant);
    }
    if (__builtin_expect(!ok, 0)) return sqrt(x);
    return __longlong_as_double((long long)res);
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

}  // namespace sl
