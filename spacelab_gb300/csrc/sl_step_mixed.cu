// sl_step_mixed.cu -- the mixed-precision form of the step (SL_MODE_MIXED).
//
// More than FP32 is kept where precision is set:
//   * FP64: positions and the whole integration (drift_kernel, shared with
//     the exact form; pass 3 in mixed_finish_kernel), the previous-step
//     distance test that chooses kin or kout, the write-step potential
//     energy of close pairs and the energy totals (far pairs' vdW potential
//     comes from a cancellation-free series in FP32, vdw_bracket);
//   * double-float (hi + lo FP32 pairs, ~48 significant bits, sl_df.cuh):
//     for pairs closer than 1.25 times the sum of their radii, the subtraction
//     r = pos[B] - pos[A] from double-float copies of the scaled positions,
//     |r|^2 and the squared gap g = (R_A + R_B)^2 - |r|^2, from which the
//     overlap is taken as g / (R_A + R_B + |r|) -- no cancellation in
//     R_A + R_B - |r|; and the per-sphere sums of the partial sums
//     (compensated, then converted to FP64).
// Everything else -- distances, the vdW coefficient, elastic, gravity,
// sliding and rolling friction, torques -- is FP32 on lengths scaled by
// 2^-len_shift (about one radius), which keeps R^6 / (S^2 T^2) far from
// FP32's range limits.  A pair at least 1.25 times its radii sum apart has a
// gap h >= (R_A + R_B) / 4, so FP32 geometry (r from the hi and lo parts)
// keeps |r|^2 - (R_A +- R_B)^2 to a few ulp, and its vdW force needs no
// square root: such pairs, nearly all of them, take a short FP32-only path.  No pair issues an FP64 instruction outside the contact
// branch and write steps: GB300's FP32 pipe is ~72x its FP64 pipe.
//
// Accumulation: the pair terms never reach memory.  A warp evaluates a
// 32 x 32 tile in a diagonal sweep -- at step k, lane b takes pair
// (row (b + k) mod 32, column b) -- so that each lane adds its column
// sphere's terms in a register and each row's running sum travels one lane
// down per step (one shuffle per component) to meet its next term; after
// the 32 steps lane l holds row l's sum.  The tile then writes one FP32
// partial per sphere and component, and mixed_finish_kernel adds a sphere's
// partials over the partner blocks in ascending order in compensated sums.
// Every order is fixed, so runs repeat bit for bit.  Large systems
// (mixed_pair_double) take a row block against two column blocks at a time
// (mixed_pair2_kernel): one shared-memory load of a row and one shuffle then
// serve two pairs.
//
// The physics follows ColliderSingleCore.cpp:104-253 term by term; only the
// arithmetic and the evaluation order differ.
#include "sl_device.cuh"
#include "sl_kernels.h"
#include "sl_df.cuh"
#include "sl_pair_mixed.cuh"

#include <type_traits>

namespace sl {

namespace {

// Row spheres of a tile in shared memory, kRowStride floats each, so that a
// warp's 16-byte loads of 32 different rows fall in distinct banks:
//   [0..3] scaled position hi x, y, z and scaled radius R,
//   [4..7] scaled position lo x, y, z and c_vdw R^3,
//   [8] the radius's lo part, [9] 1/m.
constexpr int kRowStride = 12;
constexpr int kPairWarps = 4;
constexpr int kPairCtasPerSm = 5;  // resident CTAs per SM (the launch bounds' minimum)
constexpr int kPair2CtasPerSm = 4;  // the same for two column blocks per item (128 registers, no spills)
// Two column blocks per item pay where the warps take many items each;
// with few, the longer items leave the last ones on fewer warps.
constexpr int kDoubleMinTilesPerWarp = 8;

// |pos[B] - pos[A]|^2 in FP64, the formula of the previous-step distance in
// contact_mixed (rare paths: the contact test, write-step energies).
__device__ __forceinline__ double fp64_d2(const System& s, int A, int B)
{
    const double rx = s.pos.c[0][B] - s.pos.c[0][A];
    const double ry = s.pos.c[1][B] - s.pos.c[1][A];
    const double rz = s.pos.c[2][B] - s.pos.c[2][A];
    return fma(rx, rx, fma(ry, ry, rz * rz));
}

// One warp per lower-triangular 32 x 32 block tile (X, Y), X >= Y: column
// lane b is sphere B = 32Y + b, row r is sphere A = 32X + r (A > B).  Writes
// the tile's partials f_part[c][Y][A] (sphere A's terms from block Y) and
// f_part[c][X][B] (sphere B's from block X), or on the diagonal one partial
// f_part[c][X][i] with both; contact bits to cmask[K][i]; torques of contacts
// to the float view of torqbuf, [A][B] and [B][A].
template <bool WRITE>
__global__ void __launch_bounds__(32 * kPairWarps, kPairCtasPerSm) mixed_pair_kernel(const __grid_constant__ System s)
{
    __shared__ __align__(16) float rows_all[kPairWarps][kBlock * kRowStride];
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    float* rows = rows_all[wib];
    const long long nwarps = (long long)gridDim.x * kPairWarps;
    const size_t plane = (size_t)s.npad * s.npad;  // torque planes
    const size_t pplane = (size_t)s.nb * s.npad;   // partial planes
    float* tbuf = reinterpret_cast<float*>(s.torqbuf);
    const int sh = s.len_shift;
    const float L = ldexpf(1.0f, sh);
    const float hmin_s = (float)s.mat.h_min / L;
    const float c_vdw = (float)(s.mat.Ha / 6 * 64) / L;   // dyn per unit vdw_shape
    const int nxt = (lane + 1) & (kBlock - 1);
    // write steps: close pairs out of contact whose FP64 potential is pending.
    // Their FP64 evaluation runs with every lane busy (the FP64 pipe takes a
    // warp instruction per ~64 cycles however few lanes are active)
    __shared__ int2 queue_all[WRITE ? kPairWarps : 1][WRITE ? 2 * kBlock : 1];
    int2* q = queue_all[WRITE ? wib : 0];
    int qn = 0;
    double pe = 0;
    auto flush_close = [&](int cnt) {  // pairs q[0 .. cnt), cnt <= 32; the rest move down
        if (lane < cnt) {
            const int A = q[lane].x, B = q[lane].y;
            const double d2_64 = fp64_d2(s, A, B), sum64 = s.R[A] + s.R[B];
            pe += pair_pe_fp64(s.mat, s.R[A], s.R[B], fma(sum64, sum64, -d2_64), d2_64, false, 0.0);
        }
        const int left = qn - cnt;
        const int2 e = lane < left ? q[cnt + lane] : make_int2(0, 0);
        __syncwarp();
        if (lane < left) q[lane] = e;
        __syncwarp();
        qn = left;
    };

    // Tiles: a first round in warp order, then, on plain steps, whichever
    // warp is free takes the next tile from a counter that the drift kernel
    // zeroes (the last round of a static stride leaves SMs idle); write
    // steps keep the static stride, so that their close-pair queues, and so
    // the potential energy's rounding, repeat run to run.
    long long t = (long long)blockIdx.x * kPairWarps + wib;
    for (; t < s.ntiles;) {
        int X, Y;
        tile_coords(t, X, Y);
        {
            const int i = X * kBlock + lane;  // < npad
            const float Ri = s.f_R[i];
            float* row = rows + lane * kRowStride;
            *reinterpret_cast<float4*>(row) = make_float4(s.f_pos[0][i], s.f_pos[1][i], s.f_pos[2][i], Ri);
            *reinterpret_cast<float4*>(row + 4) =
                make_float4(s.f_pos[3][i], s.f_pos[4][i], s.f_pos[5][i], c_vdw * (Ri * Ri * Ri));
            row[8] = s.f_Rlo[i];
            row[9] = s.f_inv_m[i];
        }
        __syncwarp();
        const int B = Y * kBlock + lane;
        const bool bvalid = B < s.n;
        const float bx = s.f_pos[0][B], by = s.f_pos[1][B], bz = s.f_pos[2][B];
        const float bxl = s.f_pos[3][B], byl = s.f_pos[4][B], bzl = s.f_pos[5][B];
        const float Rbs = s.f_R[B], Rblo = s.f_Rlo[B], inv_mb = s.f_inv_m[B];
        const float Rb3 = Rbs * Rbs * Rbs;
        const int nA = s.n - X * kBlock;  // rows r < nA are spheres
        pe = 0;
        df::Sum pe_far{0.0f, 0.0f};  // far pairs' vdW brackets (write steps)
        uint32_t colbits = 0;
        float ax = 0, ay = 0, az = 0;     // running sum of row (lane + k) mod 32 at step k
        float bsx = 0, bsy = 0, bsz = 0;  // sphere B's sum
        // FULL: a tile off the diagonal whose rows and columns are all spheres
        auto sweep = [&](auto full_tag) {
            constexpr bool FULL = decltype(full_tag)::value;
#pragma unroll 2
            for (int k = 0; k < kBlock; ++k) {
                const int r = (lane + k) & (kBlock - 1);
                const bool valid = FULL || (bvalid && r < nA && (X != Y || lane < r));
                const float4 q0 = *reinterpret_cast<const float4*>(rows + r * kRowStride);
                const float4 q1 = *reinterpret_cast<const float4*>(rows + r * kRowStride + 4);
                const float Ras = q0.w;
                // pairs out of contact with h = |r| - R_A - R_B above the clamp
                // h_min, in FP32 (scaled lengths): the vdW force (:205-226)
                // Ra^3 Rb^3 (h + Ra + Rb) / (S^2 T^2) along r/|r| needs no square
                // root: h + Ra + Rb = |r|, S = h (h + 2(Ra + Rb)) = |r|^2 - (Ra + Rb)^2
                // and T = S + 4 Ra Rb = |r|^2 - (Ra - Rb)^2; used for |r| >= 1.25
                // (Ra + Rb) or more, where S cancels little (far_sq)
                const float rx = (bx - q0.x) + (bxl - q1.x);
                const float ry = (by - q0.y) + (byl - q1.y);
                const float rz = (bz - q0.z) + (bzl - q1.z);
                const float d2 = fmaf(rx, rx, fmaf(ry, ry, rz * rz));
                const float sumR = Ras + Rbs, difR = Ras - Rbs;
                const float sum2 = sumR * sumR;
                const float S = d2 - sum2;
                const float T = fmaf(-difR, difR, d2);
                const float P = S * T;
                const float fr = (q1.w * Rb3) * rcp_approx(P * P);  // |F| / |r|
                float fx = fr * rx, fy = fr * ry, fz = fr * rz;
                bool contact = false;
                const bool closep = d2 < s.far_sq * sum2;
                if (valid && closep) {
                    // close pair: double-float (~48 bits, FP32 pipe) subtraction,
                    // |r|^2 and squared gap g = (R_A + R_B)^2 - |r|^2
                    const int A = X * kBlock + r;
                    const df::F2 drx = df::sub({bx, bxl}, {q0.x, q1.x});
                    const df::F2 dry = df::sub({by, byl}, {q0.y, q1.y});
                    const df::F2 drz = df::sub({bz, bzl}, {q0.z, q1.z});
                    const df::F2 dd2 = df::add(df::add(df::sqr(drx), df::sqr(dry)), df::sqr(drz));
                    const df::F2 sum = df::add({Ras, rows[r * kRowStride + 8]}, {Rbs, Rblo});
                    const df::F2 gap2 = df::sub(df::sqr(sum), dd2);
                    const float d2s = dd2.hi;
                    const float inv_dn = rsqrtf(d2s);
                    const float dist_s = d2s * inv_dn;
                    const float ovl_s = __fdividef(gap2.hi, Ras + Rbs + dist_s);
                    const float nx = drx.hi * inv_dn, ny = dry.hi * inv_dn, nz = drz.hi * inv_dn;
                    if (gap2.hi > 0.0f || (gap2.hi == 0.0f && gap2.lo > 0.0f)) {
                        contact = true;
                        colbits |= 1u << r;
                        const ContactIn in = gather_contact(s, A, B);
                        // the kin/kout test compares |r|^2 with the previous step's,
                        // both in FP64 from the FP64 positions with one formula
                        const double d2_64 = fp64_d2(s, A, B);
                        const ContactF o = contact_mixed(in, s.mat, sh, d2_64, nx, ny, nz, dist_s * L, ovl_s * L,
                                                         Ras, Rbs);
                        fx = o.fx; fy = o.fy; fz = o.fz;
                        const float ima = s.f_inv_moi[A], imb = s.f_inv_moi[B];
                        float* ta = tbuf + (size_t)A * s.npad + B;
                        float* tb = tbuf + (size_t)B * s.npad + A;
                        ta[0] = o.tax * ima; ta[plane] = o.tay * ima; ta[2 * plane] = o.taz * ima;
                        tb[0] = o.tbx * imb; tb[plane] = o.tby * imb; tb[2 * plane] = o.tbz * imb;
                        if (WRITE) {
                            const double sum64 = s.R[A] + s.R[B];
                            pe += pair_pe_fp64(s.mat, s.R[A], s.R[B], fma(sum64, sum64, -d2_64), d2_64, true, o.k);
                        }
                    } else {
                        const float hn = fmaxf(-ovl_s, hmin_s);                 // :211-215
                        const float f = c_vdw * vdw_shape(hn, Ras, Rbs);
                        fx = f * nx; fy = f * ny; fz = f * nz;
                    }
                }
                if (WRITE) {  // write steps only
                    if (valid && !closep) pe_far.add(vdw_bracket(d2, Ras, Rbs));
                    // close pairs out of contact: queued, evaluated 32 at a time
                    const bool need = valid && closep && !contact;
                    const uint32_t m = __ballot_sync(0xffffffffu, need);
                    if (m) {
                        if (need) q[qn + __popc(m & ((1u << lane) - 1u))] = make_int2(X * kBlock + r, B);
                        qn += __popc(m);
                        __syncwarp();
                        if (qn >= kBlock) flush_close(kBlock);
                    }
                }
                if (!FULL && !valid) fx = fy = fz = 0.0f;
                ax += fx; ay += fy; az += fz;
                bsx += fx; bsy += fy; bsz += fz;
                ax = __shfl_sync(0xffffffffu, ax, nxt);
                ay = __shfl_sync(0xffffffffu, ay, nxt);
                az = __shfl_sync(0xffffffffu, az, nxt);
            }
        };
        if (X != Y && (X + 1) * kBlock <= s.n)
            sweep(std::true_type{});
        else
            sweep(std::false_type{});
        // lane l now holds row l's sum; its contact bits are the transpose of
        // the lanes' column bits
        uint32_t rowbits = 0;
        if (__any_sync(0xffffffffu, colbits != 0u)) {
            for (int r = 0; r < kBlock; ++r) {
                const uint32_t wd = __ballot_sync(0xffffffffu, (colbits >> r) & 1u);
                if (lane == r) rowbits = wd;
            }
        }
        const int iA = X * kBlock + lane;
        const float ima = rows[lane * kRowStride + 9];
        float* P = s.f_part;
        if (X == Y) {  // sphere iA == B: partners j < i as A (row), j > i as B (column)
            const size_t o = (size_t)X * s.npad + iA;
            P[o] = fmaf(ima, ax, -inv_mb * bsx);
            P[o + pplane] = fmaf(ima, ay, -inv_mb * bsy);
            P[o + 2 * pplane] = fmaf(ima, az, -inv_mb * bsz);
            s.cmask[o] = rowbits | colbits;
            if (rowbits | colbits) s.contact_flag[iA] = 1;
        } else {
            const size_t oa = (size_t)Y * s.npad + iA, ob = (size_t)X * s.npad + B;
            P[oa] = ima * ax; P[oa + pplane] = ima * ay; P[oa + 2 * pplane] = ima * az;
            P[ob] = -inv_mb * bsx; P[ob + pplane] = -inv_mb * bsy; P[ob + 2 * pplane] = -inv_mb * bsz;
            s.cmask[oa] = rowbits;
            s.cmask[ob] = colbits;
            if (rowbits) s.contact_flag[iA] = 1;  // every writer stores 1
            if (colbits) s.contact_flag[B] = 1;
        }
        if (WRITE) {
            if (qn > 0 && t + nwarps >= s.ntiles) flush_close(qn);  // the warp's last tile
            pe += -s.mat.Ha / 6 * (f2d_bits(pe_far.s) + f2d_bits(pe_far.c));
            for (int off = 16; off > 0; off >>= 1) pe += __shfl_xor_sync(0xffffffffu, pe, off);
            if (lane == 0) s.pe_tile[t] = pe;
        }
        __syncwarp();
        if (WRITE) {
            t += nwarps;
        } else {
            int k = 0;
            if (lane == 0) k = atomicAdd(s.tile_counter, 1);
            t = nwarps + __shfl_sync(0xffffffffu, k, 0);
        }
    }
}

// A lane's column sphere of a tile (scaled lengths; its radius's lo part and
// 1/m are read where they are needed, which keeps two of these in registers).
struct ColSphere {
    float x, y, z, xl, yl, zl;  // position, hi and lo parts
    float R, R3;
    int B;
};

__device__ __forceinline__ ColSphere load_col(const System& s, int B)
{
    ColSphere c;
    c.B = B;
    c.x = s.f_pos[0][B]; c.y = s.f_pos[1][B]; c.z = s.f_pos[2][B];
    c.xl = s.f_pos[3][B]; c.yl = s.f_pos[4][B]; c.zl = s.f_pos[5][B];
    c.R = s.f_R[B];
    c.R3 = c.R * c.R * c.R;
    return c;
}

// One warp per work item (mixed_pair_items): row block X against one or two
// column blocks, rows A = 32X + r above columns B = 32Y + b.  With two, a
// lane holds the column spheres b of both column blocks, so that one
// shared-memory load of row r and one shuffle of its running sum serve two
// pairs.  Writes the partials f_part[c][K][i] (sphere i's terms from partner
// block K; a row sphere's terms from both column blocks go to the first, the
// second gets 0, or on the diagonal the sphere's terms as a column), contact
// bits to cmask[K][i] and torques of contacts to the float view of torqbuf,
// [A][B] and [B][A].
template <bool WRITE>
__global__ void __launch_bounds__(32 * kPairWarps, kPair2CtasPerSm) mixed_pair2_kernel(const __grid_constant__ System s)
{
    __shared__ __align__(16) float rows_all[kPairWarps][kBlock * kRowStride];
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    float* rows = rows_all[wib];
    const long long nwarps = (long long)gridDim.x * kPairWarps;
    const size_t plane = (size_t)s.npad * s.npad;  // torque planes
    const size_t pplane = (size_t)s.nb * s.npad;   // partial planes
    float* tbuf = reinterpret_cast<float*>(s.torqbuf);
    const int sh = s.len_shift;
    const float L = ldexpf(1.0f, sh);
    const float hmin_s = (float)s.mat.h_min / L;
    const float c_vdw = (float)(s.mat.Ha / 6 * 64) / L;   // dyn per unit vdw_shape
    const int nxt = (lane + 1) & (kBlock - 1);
    // write steps: close pairs out of contact whose FP64 potential is pending.
    // Their FP64 evaluation runs with every lane busy (the FP64 pipe takes a
    // warp instruction per ~64 cycles however few lanes are active)
    __shared__ int2 queue_all[WRITE ? kPairWarps : 1][WRITE ? 2 * kBlock : 1];
    int2* q = queue_all[WRITE ? wib : 0];
    int qn = 0;
    double pe = 0;
    auto flush_close = [&](int cnt) {  // pairs q[0 .. cnt), cnt <= 32; the rest move down
        if (lane < cnt) {
            const int A = q[lane].x, B = q[lane].y;
            const double d2_64 = fp64_d2(s, A, B), sum64 = s.R[A] + s.R[B];
            pe += pair_pe_fp64(s.mat, s.R[A], s.R[B], fma(sum64, sum64, -d2_64), d2_64, false, 0.0);
        }
        const int left = qn - cnt;
        const int2 e = lane < left ? q[cnt + lane] : make_int2(0, 0);
        __syncwarp();
        if (lane < left) q[lane] = e;
        __syncwarp();
        qn = left;
    };
    // lane l's bits are the rows in contact with its column sphere; returns
    // the transpose: lane l's bits are the columns in contact with row l
    auto transpose = [&](uint32_t colbits) {
        uint32_t rowbits = 0;
        if (__any_sync(0xffffffffu, colbits != 0u)) {
            for (int r = 0; r < kBlock; ++r) {
                const uint32_t wd = __ballot_sync(0xffffffffu, (colbits >> r) & 1u);
                if (lane == r) rowbits = wd;
            }
        }
        return rowbits;
    };

    // Items: a first round in warp order, then, on plain steps, whichever
    // warp is free takes the next item from a counter that the drift kernel
    // zeroes (the last round of a static stride leaves SMs idle); write
    // steps keep the static stride, so that their close-pair queues, and so
    // the potential energy's rounding, repeat run to run.
    long long t = (long long)blockIdx.x * kPairWarps + wib;
    for (; t < s.nitems;) {
        int P, Q;
        tile_coords(t >> 1, P, Q);
        const int X = 2 * P + (int)(t & 1);
        pe = 0;
        df::Sum pe_far{0.0f, 0.0f};  // far pairs' vdW brackets (write steps)
        if (X < s.nb) {
            {
                const int i = X * kBlock + lane;  // < npad
                const float Ri = s.f_R[i];
                float* row = rows + lane * kRowStride;
                *reinterpret_cast<float4*>(row) = make_float4(s.f_pos[0][i], s.f_pos[1][i], s.f_pos[2][i], Ri);
                *reinterpret_cast<float4*>(row + 4) =
                    make_float4(s.f_pos[3][i], s.f_pos[4][i], s.f_pos[5][i], c_vdw * (Ri * Ri * Ri));
                row[8] = s.f_Rlo[i];
                row[9] = s.f_inv_m[i];
            }
            __syncwarp();
            const int nA = s.n - X * kBlock;       // rows r < nA are spheres
            const bool single = P == Q && !(t & 1);  // the diagonal tile (X, X) alone
            const bool diag1 = P == Q;               // (two column blocks) the second is X
            const ColSphere c0 = load_col(s, (single ? X : 2 * Q) * kBlock + lane);

            // pairs out of contact with h = |r| - R_A - R_B above the clamp
            // h_min, in FP32 (scaled lengths): the vdW force (:205-226)
            // Ra^3 Rb^3 (h + Ra + Rb) / (S^2 T^2) along r/|r| needs no square
            // root: h + Ra + Rb = |r|, S = h (h + 2(Ra + Rb)) = |r|^2 - (Ra + Rb)^2
            // and T = S + 4 Ra Rb = |r|^2 - (Ra - Rb)^2; used for |r| >= 1.25
            // (Ra + Rb) or more, where S cancels little (far_sq).  The force
            // on the row sphere; d2 = |r|^2 and sum2 = (Ra + Rb)^2 for the test.
            auto far_force = [&](const float4& q0, const float4& q1, const ColSphere& c, float& d2, float& sum2,
                                 float& fx, float& fy, float& fz) {
                const float rx = (c.x - q0.x) + (c.xl - q1.x);
                const float ry = (c.y - q0.y) + (c.yl - q1.y);
                const float rz = (c.z - q0.z) + (c.zl - q1.z);
                d2 = fmaf(rx, rx, fmaf(ry, ry, rz * rz));
                const float sumR = q0.w + c.R, difR = q0.w - c.R;
                sum2 = sumR * sumR;
                const float S = d2 - sum2;
                const float T = fmaf(-difR, difR, d2);
                const float Pst = S * T;
                const float fr = (q1.w * c.R3) * rcp_approx(Pst * Pst);  // |F| / |r|
                fx = fr * rx; fy = fr * ry; fz = fr * rz;
            };
            // close pair (row r, column sphere c): double-float (~48 bits, FP32
            // pipe) subtraction, |r|^2 and squared gap g = (R_A + R_B)^2 - |r|^2,
            // then the contact branch or the clamped vdW; true in contact
            auto close_pair = [&](int r, const float4& q0, const float4& q1, const ColSphere& c, uint32_t& bits,
                                  float& fx, float& fy, float& fz) {
                const int A = X * kBlock + r, B = c.B;
                const float Ras = q0.w;
                const df::F2 drx = df::sub({c.x, c.xl}, {q0.x, q1.x});
                const df::F2 dry = df::sub({c.y, c.yl}, {q0.y, q1.y});
                const df::F2 drz = df::sub({c.z, c.zl}, {q0.z, q1.z});
                const df::F2 dd2 = df::add(df::add(df::sqr(drx), df::sqr(dry)), df::sqr(drz));
                const df::F2 sum = df::add({Ras, rows[r * kRowStride + 8]}, {c.R, s.f_Rlo[B]});
                const df::F2 gap2 = df::sub(df::sqr(sum), dd2);
                const float d2s = dd2.hi;
                const float inv_dn = rsqrtf(d2s);
                const float dist_s = d2s * inv_dn;
                const float ovl_s = __fdividef(gap2.hi, Ras + c.R + dist_s);
                const float nx = drx.hi * inv_dn, ny = dry.hi * inv_dn, nz = drz.hi * inv_dn;
                if (gap2.hi > 0.0f || (gap2.hi == 0.0f && gap2.lo > 0.0f)) {
                    bits |= 1u << r;
                    const ContactIn in = gather_contact(s, A, B);
                    // the kin/kout test compares |r|^2 with the previous step's,
                    // both in FP64 from the FP64 positions with one formula
                    const double d2_64 = fp64_d2(s, A, B);
                    const ContactF o = contact_mixed(in, s.mat, sh, d2_64, nx, ny, nz, dist_s * L, ovl_s * L, Ras,
                                                     c.R);
                    fx = o.fx; fy = o.fy; fz = o.fz;
                    const float ima = s.f_inv_moi[A], imb = s.f_inv_moi[B];
                    float* ta = tbuf + (size_t)A * s.npad + B;
                    float* tb = tbuf + (size_t)B * s.npad + A;
                    ta[0] = o.tax * ima; ta[plane] = o.tay * ima; ta[2 * plane] = o.taz * ima;
                    tb[0] = o.tbx * imb; tb[plane] = o.tby * imb; tb[2 * plane] = o.tbz * imb;
                    if (WRITE) {
                        const double sum64 = s.R[A] + s.R[B];
                        pe += pair_pe_fp64(s.mat, s.R[A], s.R[B], fma(sum64, sum64, -d2_64), d2_64, true, o.k);
                    }
                    return true;
                }
                const float hn = fmaxf(-ovl_s, hmin_s);                 // :211-215
                const float f = c_vdw * vdw_shape(hn, Ras, c.R);
                fx = f * nx; fy = f * ny; fz = f * nz;
                return false;
            };
            // write steps only: the far pair's vdW bracket, or the close pair
            // out of contact queued for its FP64 potential (32 at a time)
            auto write_terms = [&](bool valid, bool closep, bool contact, float d2, float Ras, const ColSphere& c,
                                   int r) {
                if (valid && !closep) pe_far.add(vdw_bracket(d2, Ras, c.R));
                const bool need = valid && closep && !contact;
                const uint32_t m = __ballot_sync(0xffffffffu, need);
                if (m) {
                    if (need) q[qn + __popc(m & ((1u << lane) - 1u))] = make_int2(X * kBlock + r, c.B);
                    qn += __popc(m);
                    __syncwarp();
                    if (qn >= kBlock) flush_close(kBlock);
                }
            };

            uint32_t bits0 = 0, bits1 = 0;      // contact rows of the lane's column spheres
            float ax = 0, ay = 0, az = 0;       // running sum of row (lane + k) mod 32 at step k
            float b0x = 0, b0y = 0, b0z = 0;    // column sphere sums
            float b1x = 0, b1y = 0, b1z = 0;
            const int iA = X * kBlock + lane;
            const float ima = rows[lane * kRowStride + 9];
            float* Pt = s.f_part;
            if (single) {
#pragma unroll 2
                for (int k = 0; k < kBlock; ++k) {
                    const int r = (lane + k) & (kBlock - 1);
                    const bool valid = r < nA && lane < r;
                    const float4 q0 = *reinterpret_cast<const float4*>(rows + r * kRowStride);
                    const float4 q1 = *reinterpret_cast<const float4*>(rows + r * kRowStride + 4);
                    float d2, sum2, fx, fy, fz;
                    far_force(q0, q1, c0, d2, sum2, fx, fy, fz);
                    const bool closep = d2 < s.far_sq * sum2;
                    bool contact = false;
                    if (valid && closep) contact = close_pair(r, q0, q1, c0, bits0, fx, fy, fz);
                    if (WRITE) write_terms(valid, closep, contact, d2, q0.w, c0, r);
                    if (!valid) fx = fy = fz = 0.0f;
                    ax += fx; ay += fy; az += fz;
                    b0x += fx; b0y += fy; b0z += fz;
                    ax = __shfl_sync(0xffffffffu, ax, nxt);
                    ay = __shfl_sync(0xffffffffu, ay, nxt);
                    az = __shfl_sync(0xffffffffu, az, nxt);
                }
                // lane l now holds row l's sum; sphere iA is both row and column
                const uint32_t rowbits = transpose(bits0);
                const size_t o = (size_t)X * s.npad + iA;
                Pt[o] = fmaf(ima, ax, -ima * b0x);
                Pt[o + pplane] = fmaf(ima, ay, -ima * b0y);
                Pt[o + 2 * pplane] = fmaf(ima, az, -ima * b0z);
                s.cmask[o] = rowbits | bits0;
                if (rowbits | bits0) s.contact_flag[iA] = 1;
            } else {
                const ColSphere c1 = load_col(s, (2 * Q + 1) * kBlock + lane);
                // FULL: both column blocks below X and every row a sphere (the
                // column blocks below X are full)
                auto sweep = [&](auto full_tag) {
                    constexpr bool FULL = decltype(full_tag)::value;
#pragma unroll 2
                    for (int k = 0; k < kBlock; ++k) {
                        const int r = (lane + k) & (kBlock - 1);
                        const bool v0 = FULL || r < nA;
                        const bool v1 = FULL || (r < nA && (!diag1 || lane < r));
                        const float4 q0 = *reinterpret_cast<const float4*>(rows + r * kRowStride);
                        const float4 q1 = *reinterpret_cast<const float4*>(rows + r * kRowStride + 4);
                        float d20, s20, f0x, f0y, f0z, d21, s21, f1x, f1y, f1z;
                        far_force(q0, q1, c0, d20, s20, f0x, f0y, f0z);
                        far_force(q0, q1, c1, d21, s21, f1x, f1y, f1z);
                        const bool cl0 = d20 < s.far_sq * s20, cl1 = d21 < s.far_sq * s21;
                        bool ct0 = false, ct1 = false;
                        if (v0 && cl0) ct0 = close_pair(r, q0, q1, c0, bits0, f0x, f0y, f0z);
                        if (v1 && cl1) ct1 = close_pair(r, q0, q1, c1, bits1, f1x, f1y, f1z);
                        if (WRITE) {
                            write_terms(v0, cl0, ct0, d20, q0.w, c0, r);
                            write_terms(v1, cl1, ct1, d21, q0.w, c1, r);
                        }
                        if (!FULL) {
                            if (!v0) f0x = f0y = f0z = 0.0f;
                            if (!v1) f1x = f1y = f1z = 0.0f;
                        }
                        ax += f0x + f1x; ay += f0y + f1y; az += f0z + f1z;
                        b0x += f0x; b0y += f0y; b0z += f0z;
                        b1x += f1x; b1y += f1y; b1z += f1z;
                        ax = __shfl_sync(0xffffffffu, ax, nxt);
                        ay = __shfl_sync(0xffffffffu, ay, nxt);
                        az = __shfl_sync(0xffffffffu, az, nxt);
                    }
                };
                if (!diag1 && (X + 1) * kBlock <= s.n)
                    sweep(std::true_type{});
                else
                    sweep(std::false_type{});
                // lane l now holds row l's sum over both column blocks
                const uint32_t rb0 = transpose(bits0), rb1 = transpose(bits1);
                const size_t oa0 = (size_t)(2 * Q) * s.npad + iA, oa1 = oa0 + s.npad;
                const size_t ob0 = (size_t)X * s.npad + c0.B, ob1 = (size_t)X * s.npad + c1.B;
                Pt[oa0] = ima * ax; Pt[oa0 + pplane] = ima * ay; Pt[oa0 + 2 * pplane] = ima * az;
                const float imb0 = s.f_inv_m[c0.B], imb1 = s.f_inv_m[c1.B];
                Pt[ob0] = -imb0 * b0x; Pt[ob0 + pplane] = -imb0 * b0y; Pt[ob0 + 2 * pplane] = -imb0 * b0z;
                s.cmask[oa0] = rb0;
                s.cmask[ob0] = bits0;
                if (diag1) {  // column sphere c1 is the row sphere iA: its partners after it in block X
                    Pt[oa1] = -imb1 * b1x; Pt[oa1 + pplane] = -imb1 * b1y; Pt[oa1 + 2 * pplane] = -imb1 * b1z;
                    s.cmask[oa1] = rb1 | bits1;
                } else {
                    Pt[oa1] = 0.0f; Pt[oa1 + pplane] = 0.0f; Pt[oa1 + 2 * pplane] = 0.0f;
                    Pt[ob1] = -imb1 * b1x; Pt[ob1 + pplane] = -imb1 * b1y; Pt[ob1 + 2 * pplane] = -imb1 * b1z;
                    s.cmask[oa1] = rb1;
                    s.cmask[ob1] = bits1;
                }
                if (rb0 | rb1) s.contact_flag[iA] = 1;  // every writer stores 1
                if (bits0) s.contact_flag[c0.B] = 1;
                if (bits1) s.contact_flag[c1.B] = 1;
            }
        }
        if (WRITE) {
            if (qn > 0 && t + nwarps >= s.nitems) flush_close(qn);  // the warp's last item
            pe += -s.mat.Ha / 6 * (f2d_bits(pe_far.s) + f2d_bits(pe_far.c));
            for (int off = 16; off > 0; off >>= 1) pe += __shfl_xor_sync(0xffffffffu, pe, off);
            if (lane == 0) s.pe_tile[t] = pe;
        }
        __syncwarp();
        if (WRITE) {
            t += nwarps;
        } else {
            int k = 0;
            if (lane == 0) k = atomicAdd(s.tile_counter, 1);
            t = nwarps + __shfl_sync(0xffffffffu, k, 0);
        }
    }
}

constexpr int kFinSlices = 8;

// Per-sphere totals, then pass 3.  Block = 32 spheres (lanes) x kFinSlices
// warps; warp w adds partner blocks [nb w / S, nb (w+1) / S) of its lane's
// sphere: the force partials f_part[c][K][i] (coalesced loads along i) and
// the torque terms of contact partners (bits of cmask[K][i], ascending), all
// in compensated double-float sums.  Warp c < 3 then adds component c's
// slices in order, still on the FP32 pipe, and integrates it in FP64
// (ColliderSingleCore.cpp:263-267): a handful of FP64 instructions per warp,
// which GB300 issues at one per 64 cycles or so.
__global__ void __launch_bounds__(32 * kFinSlices) mixed_finish_kernel(const __grid_constant__ System s)
{
    __shared__ float fs[kFinSlices][12][kBlock];  // (s, c) of force x, y, z, then of torque x, y, z
    const int lane = threadIdx.x & 31;
    const int w = threadIdx.x >> 5;
    const int i = blockIdx.x * kBlock + lane;  // < npad
    const int K0 = (int)((long long)s.nb * w / kFinSlices);
    const int K1 = (int)((long long)s.nb * (w + 1) / kFinSlices);
    const size_t pplane = (size_t)s.nb * s.npad;
    const size_t plane = (size_t)s.npad * s.npad;
    const float* p = s.f_part + i;
    const uint32_t* mk = s.cmask + i;
    // contact words only for spheres with a contact this step (few)
    const bool any_contact = i < s.n && s.contact_flag[i] != 0;
    const float* tb = reinterpret_cast<const float*>(s.torqbuf) + (size_t)i * s.npad;
    df::Sum f[3] = {{0.0f, 0.0f}, {0.0f, 0.0f}, {0.0f, 0.0f}};
    df::Sum tq[3] = {{0.0f, 0.0f}, {0.0f, 0.0f}, {0.0f, 0.0f}};
    auto torques = [&](uint32_t wd, int K) {
        while (wd) {
            const int j = K * kBlock + __ffs(wd) - 1;
            wd &= wd - 1;
#pragma unroll
            for (int c = 0; c < 3; ++c) tq[c].add(tb[j + c * plane]);
        }
    };
    constexpr int U = 8;  // loads in flight per array
    int K = K0;
    for (; K + U <= K1; K += U) {
        float v[3][U];
        uint32_t m[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const size_t o = (size_t)(K + u) * s.npad;
#pragma unroll
            for (int c = 0; c < 3; ++c) v[c][u] = __ldcs(p + o + c * pplane);
            m[u] = any_contact ? __ldcs(mk + o) : 0u;
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
#pragma unroll
            for (int c = 0; c < 3; ++c) f[c].add(v[c][u]);
            torques(m[u], K + u);
        }
    }
    for (; K < K1; ++K) {
        const size_t o = (size_t)K * s.npad;
#pragma unroll
        for (int c = 0; c < 3; ++c) f[c].add(__ldcs(p + o + c * pplane));
        torques(any_contact ? __ldcs(mk + o) : 0u, K);
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        fs[w][2 * c][lane] = f[c].s;
        fs[w][2 * c + 1][lane] = f[c].c;
        fs[w][6 + 2 * c][lane] = tq[c].s;
        fs[w][7 + 2 * c][lane] = tq[c].c;
    }
    __syncthreads();
    if (w >= 3 || i >= s.n) return;
    const int c = w;
    df::Sum F{0.0f, 0.0f}, Q{0.0f, 0.0f};
#pragma unroll
    for (int ww = 0; ww < kFinSlices; ++ww) {
        F.add(fs[ww][2 * c][lane]);
        F.add(fs[ww][2 * c + 1][lane]);
        Q.add(fs[ww][6 + 2 * c][lane]);
        Q.add(fs[ww][7 + 2 * c][lane]);
    }
    const double acc = f2d_bits(F.s) + f2d_bits(F.c);
    const double aacc = f2d_bits(Q.s) + f2d_bits(Q.c);
    const double dt = s.sc->dt;
    const double v = s.velh.c[c][i] + (.5 * acc) * dt;    // :265
    const double wv = s.wh.c[c][i] + (.5 * aacc) * dt;   // :266
    s.acc.c[c][i] = acc;
    s.aacc.c[c][i] = aacc;
    s.vel.c[c][i] = v;
    s.w.c[c][i] = wv;
    if (!isfinite(v) || !isfinite(wv) || !isfinite(s.pos.c[c][i])) atomicOr(s.status, 1u);
}

}  // namespace

bool mixed_pair_double(int nb, int num_sms)
{
    const long long ntiles = (long long)nb * (nb + 1) / 2;
    const long long warps = (long long)num_sms * kPair2CtasPerSm * kPairWarps;
    return ntiles >= kDoubleMinTilesPerWarp * warps;
}

void launch_step_mixed(const System& s, bool write, int num_sms, cudaStream_t st, StepTimers* tm)
{
    launch_drift(s, st);
    if (tm) cudaEventRecord(tm->ev[0], st);
    long long want = (s.nitems + kPairWarps - 1) / kPairWarps;
    // one wave of persistent warps
    long long cap = (long long)num_sms * (s.pair_double ? kPair2CtasPerSm : kPairCtasPerSm);
    const int pb = (int)(want < cap ? want : cap);
    if (s.pair_double) {
        if (write)
            mixed_pair2_kernel<true><<<pb, 32 * kPairWarps, 0, st>>>(s);
        else
            mixed_pair2_kernel<false><<<pb, 32 * kPairWarps, 0, st>>>(s);
    } else {
        if (write)
            mixed_pair_kernel<true><<<pb, 32 * kPairWarps, 0, st>>>(s);
        else
            mixed_pair_kernel<false><<<pb, 32 * kPairWarps, 0, st>>>(s);
    }
    if (tm) cudaEventRecord(tm->ev[1], st);
    mixed_finish_kernel<<<s.nb, 32 * kFinSlices, 0, st>>>(s);
    if (tm) cudaEventRecord(tm->ev[2], st);
    if (write) launch_energy(s, st);
}

}  // namespace sl
