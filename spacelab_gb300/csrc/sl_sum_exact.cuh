// sl_sum_exact.cuh -- a running FP64 sum, s <- RN(s + t) term after term,
// computed on the integer pipe and bit-identical to the FP64 additions.
//
// Purpose: the exact row sums add n terms in a fixed order, one dependent
// FP64 add after another, and on GB300 a dependent FP64 add costs 64-76
// cycles (one narrow FP64 unit per SM).  Here the dependent part of an
// addition is a few integer adds and shifts.  Measured on GB300 (N=5000
// row sums), the whole addition costs ~56 instructions, ~49 of them on the
// ALU pipe, which issues a warp instruction every other cycle: ~160 cycles
// per addition with one warp per scheduler, so the FP64 unit stays the
// faster choice there (sl_set_rowsum selects either; the sums are equal).
//
// Representation.  The running sum is held in a fixed-point frame: p is the
// binade of the sum (its biased FP64 exponent), and the frame's unit is
// 2^(p - 1084), so that a sum of binade p has its leading bit at bit 61 of a
// 64-bit integer and its last significand bit at bit 9.  The state keeps
// r8 = R >> 8, R the correctly rounded sum in that frame (a multiple of 2^9,
// |R| in [2^61, 2^62]); q = p - 896 (the FP32-biased exponent).
//
// One addition (step):
//   1. Predict the binade of the new sum from an FP32 "shadow" sum s32 += t,
//      off the critical path: qn = exponent of s32.
//   2. Move the old sum to the new frame: M = r8 << (q + 8 - qn), exact for
//      a binade change of -1..+8 (sh in [0, 9]); r8 is even, so M is even.
//   3. Align the term: W = significand << 10 (leading bit 62), T = W >> c
//      with c = p + 1 - e_t >= 1, and the sticky bit (bits shifted out) ORed
//      into bit 0 -- "jamming": since M is even, the jammed sum X is odd
//      whenever bits were lost, lies on the same side of every even integer
//      as the exact sum, and can never be a tie.  Zero and subnormal terms
//      take c >= 63 and act as a nonzero term below half an ulp, which leaves
//      the sum unchanged, as IEEE addition does.
//   4. X = M +/- T (64-bit two's complement), then round to nearest even at
//      bit 9: R = ((X + 0xFF + bit9(X)) >> 9) << 9.
//   5. Check that X's leading bit is bit 61, i.e. that the prediction was
//      right.  With |M| <= 2^63 and |T| < 2^62 a wrapped 64-bit X always has
//      its leading bit at 62 or 63, so the check also rules out overflow.
// When the checks hold (sh in [0, 9], c >= 1, X in binade 61) the rounding
// position is the IEEE one for the exact sum's binade, so R is RN(s + t).
// Otherwise the step's result is meaningless and `bad` is set; the caller
// then repeats the whole chunk of terms with FP64 additions from the sum it
// saved at the chunk's start (to_double), so results never depend on
// which path ran.  Tested bit for bit against hardware FP64 additions in
// tests/test_sum_exact.py (random, adversarial and cancelling sequences).
#pragma once
#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define SL_XS_FN __host__ __device__ __forceinline__
#else
#define SL_XS_FN inline
#endif

namespace sl {
namespace xs {

constexpr int kBiasShift = 896;      // FP64 exponent bias - FP32 exponent bias
constexpr int kNoFrame = -100000;    // q of a sum the frame cannot hold (0, subnormal, Inf, NaN)

SL_XS_FN uint32_t f2u(float f)
{
#ifdef __CUDA_ARCH__
    return __float_as_uint(f);
#else
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return u;
#endif
}
SL_XS_FN float u2f(uint32_t u)
{
#ifdef __CUDA_ARCH__
    return __uint_as_float(u);
#else
    float f;
    std::memcpy(&f, &u, 4);
    return f;
#endif
}
SL_XS_FN uint64_t d2u(double d)
{
#ifdef __CUDA_ARCH__
    return (uint64_t)__double_as_longlong(d);
#else
    uint64_t u;
    std::memcpy(&u, &d, 8);
    return u;
#endif
}
SL_XS_FN double u2d(uint64_t u)
{
#ifdef __CUDA_ARCH__
    return __longlong_as_double((long long)u);
#else
    double d;
    std::memcpy(&d, &u, 8);
    return d;
#endif
}

// A running sum in the frame form.
struct Run {
    int64_t r8;  // R >> 8 (even); R = the sum in units of 2^(q + kBiasShift - 1084)
    int q;       // binade, FP32-biased; kNoFrame when the sum is 0, subnormal or not finite
};

// The FP64 sum a frame state stands for (q != kNoFrame).  |R| = m 2^9 with
// m in [2^52, 2^53]; the value is m 2^(p - 1075): exponent field p, or p + 1
// when m = 2^53, both given by ((p - 1) << 52) + m.
SL_XS_FN double to_double(const Run& r)
{
    const uint64_t neg = (uint64_t)(r.r8 >> 63);
    const uint64_t m = (((uint64_t)r.r8 ^ neg) - neg) >> 1;
    const uint64_t p = (uint64_t)(r.q + kBiasShift);
    return u2d((((p - 1) << 52) + m) | (neg << 63));
}

// The frame state of an FP64 sum; kNoFrame for 0, subnormals, Inf and NaN.
SL_XS_FN Run from_double(double s)
{
    const uint64_t b = d2u(s);
    const int p = (int)((b >> 52) & 0x7ff);
    Run r;
    if (p == 0 || p == 0x7ff) {
        r.r8 = 0;
        r.q = kNoFrame;
        return r;
    }
    const int64_t m = (int64_t)(((b & 0xfffffffffffffull) | (1ull << 52)) << 1);
    r.r8 = (b >> 63) ? -m : m;
    r.q = p - kBiasShift;
    return r;
}

// FP32 approximation of the sum (the shadow's value at a chunk's start),
// good to ~2^-21 relative; only the binade predictions depend on it.
SL_XS_FN float shadow_of(const Run& r)
{
    const uint32_t hi = (uint32_t)((uint64_t)r.r8 >> 32);
    const uint32_t sgn = (uint32_t)((int32_t)hi >> 31);
    const uint32_t a = hi ^ sgn;  // |r8| >> 32 (one's complement for negative sums)
    const uint32_t frac = (a << 2) & 0x7fffffu;
    return u2f(frac | ((uint32_t)r.q << 23) | (sgn & 0x80000000u));
}

// FP32 approximation of an FP64 term from its high word: exponent rebiased,
// mantissa truncated to 20 bits.  Terms outside FP32's normal range give a
// meaningless value, which can only cost a failed prediction.
SL_XS_FN float term_f32(uint32_t thi)
{
    return u2f(((thi << 3) - 0xC0000000u) | (thi & 0x80000000u));
}

// One addition s <- RN(s + t) in the frame of binade qn (FP32-biased); see
// the header.  `bad` collects the failures of the fast path's conditions
// (nonzero: the result must not be used).  Any qn is safe: a wrong one
// only sets `bad`.
SL_XS_FN void step_in(Run& r, int qn, uint32_t& bad, uint64_t tb)
{
    const uint32_t thi = (uint32_t)(tb >> 32);
    // 2. the old sum in the new frame
    const int sh = r.q + 8 - qn;
    const uint64_t m = (uint64_t)r.r8 << (sh & 31);
    // 3. the term in the new frame, with the sticky bit jammed into bit 0
    const int et = (int)((thi >> 20) & 0x7ffu);
    const int c = qn + kBiasShift + 1 - et;
    const int cc = c < 63 ? (c > 0 ? c : 0) : 63;
    const uint64_t w = ((tb << 10) & 0x3fffffffffffffffull) | (1ull << 62);
    const uint64_t tt = w >> cc;
    const uint64_t st = (tt << cc) != w ? 1ull : 0ull;
    const uint64_t sg = (uint64_t)((int64_t)tb >> 63);
    // 4. exact sum (mod 2^64) and round to nearest even at bit 9
    const uint64_t x = m + ((tt | st) ^ sg) - sg;
    const uint64_t y = x + 0xffull + ((x >> 9) & 1ull);
    r.r8 = (int64_t)(((int64_t)y >> 9) << 1);
    r.q = qn;
    // 5. the conditions under which r is RN(s + t)
    const uint32_t xh = (uint32_t)(x >> 32);
    const uint32_t a = xh ^ (uint32_t)((int32_t)xh >> 31);
    bad |= (uint32_t)((a >> 29) != 1u) | (uint32_t)((unsigned)sh > 9u) | (uint32_t)(c < 1);
}

// One addition with the binade predicted by the shadow sum s32 (step 1).
SL_XS_FN void step(Run& r, float& s32, uint32_t& bad, uint64_t tb)
{
    s32 = s32 + term_f32((uint32_t)(tb >> 32));
    step_in(r, (int)((f2u(s32) >> 23) & 0xffu), bad, tb);
}

}  // namespace xs
}  // namespace sl
