// sl_device.cuh -- device-side data layout and arithmetic helpers shared by
// the step kernels.
//
// HBM layout of one system (all arrays are structure-of-arrays, padded to
// npad = ceil(n / 32) * 32 spheres so that every 32-sphere block is whole):
//   pos, prev, vel, velh, w, wh, acc, aacc   [3][npad] doubles (x, y, z rows)
//   R, m, moi                                [npad]
//   twoR = 2R, fourR = 4R                    exact power-of-two scalings
//   cR3  = ((Ha/6*64)*R)*R*R                 the sphere-A prefix of the vdW
//                                            coefficient chain
//   inv_m = RN(1/m), inv_moi = RN(1/moi)     correctly rounded reciprocals
//   pairbuf[3][npad][npad]                   per-pair force contributions,
//                                            row s holds the terms that sphere
//                                            s adds to acc[s] (scratch)
//   torqbuf[3][npad][npad]                   per-pair torque contributions,
//                                            written only for contacts
//   cmask[npad][nb]                          contact bit per (s, 32-block);
//                                            the mixed form stores it
//                                            [nb][npad] (block-major)
//   f_part[3][nb][npad]                      double-float mixed form: per-tile
//                                            FP32 partial sums (pairbuf unused)
//   part64[3][nb][npad]                      FP64-accumulating mixed form:
//                                            per-tile FP64 force partials
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace sl {

constexpr int kBlock = 32;  // spheres per pair tile edge (one warp lane each)

struct Material {
    double G, Ha, u_s, u_r, h_min;
};

// Per-step scalars live in device memory so that captured CUDA graphs stay
// valid when the host changes dt or the spring constants.
struct Scalars {
    double dt, kin, kout;
};

struct Vec3Soa {
    double* c[3];
};

struct System {
    int n, npad, nb;
    long long ntiles;  // nb * (nb + 1) / 2 lower-triangular block tiles
    long long nitems;  // pair-kernel work items, one pe_tile entry each: ntiles, or
                       // mixed_pair_items(nb) where pair_double is set
    int pair_double;   // mixed form: two column blocks per work item
    Vec3Soa pos, prev, vel, velh, w, wh, acc, aacc;
    double *R, *m, *moi, *twoR, *fourR, *cR3;
    unsigned long long* rm;  // 64-bit fixed-point reciprocal significand of m (recip_sig)
    double* inv_moi;
    double* pairbuf;      // [3][npad][npad]
    double* torqbuf;      // [3][npad][npad]
    uint32_t* cmask;      // [npad][nb]
    double* pe_tile;      // [nitems]
    double* red;          // [kRedBlocks][8] energy partials
    double* energy;       // [8] PE, KE, mom xyz, L xyz
    unsigned int* status; // error bits (see SL_ERR_* in spacelab_gpu.h)
    const Scalars* sc;
    Material mat;
    // mixed-precision form: per-sphere FP32 constants in lengths scaled by
    // 2^-len_shift (a power of two near the largest radius); NULL otherwise
    float *f_R, *f_inv_m, *f_inv_moi;
    // and double-float (hi + lo) copies of the scaled radii's low parts and
    // of the scaled positions (x, y, z hi, then x, y, z lo), the latter
    // written by the drift kernel every step
    float *f_Rlo, *f_pos[6];
    // the double-float mixed form's per-tile partial sums [3][nb][npad]
    // (FP32): entry (c, K, i) is component c of sphere i's acceleration terms
    // from the partners in 32-sphere block K
    float* f_part;
    // the FP64-accumulating mixed form's per-tile partial sums [3][nb][npad]
    // (FP64): entry (c, K, i) is component c of the force on sphere i from
    // the partners in 32-sphere block K
    double* part64;
    // the pair kernels' tile counters, one per pair phase (NULL: static
    // tile stride), and, mixed forms, per sphere a flag set when any of its
    // pairs is in contact (both zeroed by the drift kernel)
    int* tile_counter;
    int* contact_flag;
    int len_shift;
    // mixed form: squared separation factor of the far-pair paths
    // (far_threshold_sq in sl_pair_mixed.cuh)
    float far_sq;
};

// Operands of a pair's contact branch beyond positions and radii (the
// contact branch is rare: O(N) of the O(N^2) pairs, so they are gathered
// from global memory when needed).
struct ContactIn {
    double prevA[3], prevB[3];  // positions of the previous step
    double wA[3], wB[3], vA[3], vB[3];
    double mA, mB, kin, kout;
};

__device__ __forceinline__ ContactIn gather_contact(const System& s, int A, int B)
{
    ContactIn in;
    for (int c = 0; c < 3; ++c) {
        in.prevA[c] = s.prev.c[c][A]; in.prevB[c] = s.prev.c[c][B];
        in.wA[c] = s.w.c[c][A]; in.wB[c] = s.w.c[c][B];
        in.vA[c] = s.vel.c[c][A]; in.vB[c] = s.vel.c[c][B];
    }
    in.mA = s.m[A]; in.mB = s.m[B];
    in.kin = s.sc->kin; in.kout = s.sc->kout;
    return in;
}

// Exact float -> double (IEEE, bit manipulation on the integer pipe).
// Float subnormals flush to a signed zero; Inf/NaN keep their class.
__device__ __forceinline__ double f2d_bits(float f)
{
    const unsigned u = __float_as_uint(f);
    const unsigned long long sign = (unsigned long long)(u >> 31) << 63;
    const unsigned e = (u >> 23) & 0xffu;
    const unsigned long long m = u & 0x7fffffu;
    const unsigned long long ed = (e == 0xffu) ? 0x7ffull : (unsigned long long)(e + 896u);
    const unsigned long long body = (e == 0u) ? 0ull : ((ed << 52) | (m << 29));  // select, no branch
    return __longlong_as_double((long long)(sign | body));
}

// RN-even double -> float of x * 2^-shift (bit manipulation on the integer
// pipe; an exact power-of-two scaling folded into the exponent).  Results
// below the float normal range flush to a signed zero, above it give Inf.
__device__ __forceinline__ float d2f_bits(double x, int shift)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned sign = (unsigned)(b >> 63) << 31;
    const int e = (int)((b >> 52) & 0x7ffull);
    if (e == 0) return __uint_as_float(sign);
    const int fe = e - 1023 + 127 - shift;
    if (fe <= 0) return __uint_as_float(sign);
    if (fe >= 255 || e == 0x7ff) return __uint_as_float(sign | 0x7f800000u);
    const unsigned long long mant = b & 0xfffffffffffffull;
    const unsigned m23 = (unsigned)(mant >> 29);
    const unsigned rem = (unsigned)(mant & 0x1fffffffull);
    unsigned r = ((unsigned)fe << 23) | m23;
    r += (rem > 0x10000000u || (rem == 0x10000000u && (m23 & 1u))) ? 1u : 0u;  // may carry into Inf
    return __uint_as_float(sign | r);
}

// Correctly rounded quotient a / b given y = RN(1/b) (b > 0, normal range).
// Two residual corrections after q0 = RN(a*y), following Markstein's
// theorem for FMA-based division (P. Markstein, "Computation of elementary
// functions on the IBM RISC System/6000 processor", IBM J. Res. Dev. 34(1),
// 1990; see also Muller et al., Handbook of Floating-Point Arithmetic,
// ch. "Division"):
//   q1 = q0 + (a - b q0) y   is a faithful rounding of a/b,
//   q2 = q1 + (a - b q1) y   with exact residual, equals RN(a/b) because
//   |q1 + r1 y - a/b| <= |a/b - q1| * |1 - b y| < (ulp/2 + d) u, and a
//   quotient of two 53-bit numbers is more than 2^-54 ulp from any midpoint.
// Five FP64 pipe operations instead of a full division; tested bit-for-bit
// against IEEE division in tests/test_gpu_division.py.
__device__ __forceinline__ double div_by_recip(double a, double b, double y)
{
    const double q0 = a * y;
    const double r0 = fma(-b, q0, a);
    const double q1 = fma(r0, y, q0);
    const double r1 = fma(-b, q1, a);
    return fma(r1, y, q1);
}

// Lower-triangular tile index t -> (X, Y), X >= Y, t = X(X+1)/2 + Y.
// Work items of the mixed pair kernel: the lower-triangular 32 x 32 block
// tiles grouped in 64 x 64 macro tiles (P, Q), P >= Q, of block rows 2P and
// 2P + 1 and block columns 2Q and 2Q + 1.  Item 2m + h of macro tile m is row
// block X = 2P + h against column blocks 2Q and 2Q + 1, both below X when
// P > Q; when P == Q, h = 0 is the diagonal tile (X, X) alone and h = 1 takes
// the tiles (X, X - 1) and (X, X).  An item whose row block X >= nb is empty.
__host__ __device__ inline long long mixed_pair_items(int nb)
{
    const long long m = (nb + 1) / 2;
    return m * (m + 1);
}

__device__ __forceinline__ void tile_coords(long long t, int& X, int& Y)
{
    // FP32 estimate (the FP64 pipe is slow), corrected exactly below
    long long x = (long long)((sqrtf(8.0f * (float)t + 1.0f) - 1.0f) * 0.5f);
    if (x < 0) x = 0;
    while (x * (x + 1) / 2 > t) --x;
    while ((x + 1) * (x + 2) / 2 <= t) ++x;
    X = (int)x;
    Y = (int)(t - x * (x + 1) / 2);
}

}  // namespace sl
