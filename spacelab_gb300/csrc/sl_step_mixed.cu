// sl_step_mixed.cu -- the mixed-precision form of the step (SL_MODE_MIXED).
//
// More than FP32 is kept where precision is set:
//   * FP64: positions and the whole integration (drift_kernel, shared with
//     the exact form; pass 3 in the row sums), the previous-step distance
//     test that chooses kin or kout, the write-step potential energy per
//     pair and the energy totals;
//   * double-float (hi + lo FP32 pairs, ~48 significant bits, sl_df.cuh):
//     the pair subtraction r = pos[B] - pos[A] from double-float copies of
//     the scaled positions, |r|^2 and the squared gap
//     g = (R_A + R_B)^2 - |r|^2, from which the overlap is taken as
//     g / (R_A + R_B + |r|) -- no cancellation in R_A + R_B - |r|; and the
//     per-sphere sums of the FP32 pair terms (compensated, in ascending
//     partner order, then converted to FP64).
// Everything else -- distances, the vdW coefficient, elastic, gravity,
// sliding and rolling friction, torques -- is FP32 on lengths scaled by
// 2^-len_shift (about one radius), which keeps R^6 / (S^2 T^2) far from
// FP32's range limits.  The non-contact pair path thus issues no FP64
// instruction: GB300's FP32 pipe is ~72x its FP64 pipe.
// The physics follows ColliderSingleCore.cpp:104-253 term by term; only the
// arithmetic and the evaluation order differ.
#include "sl_device.cuh"
#include "sl_kernels.h"
#include "sl_df.cuh"
#include "sl_pair_mixed.cuh"

namespace sl {

namespace {

struct ABlockMixed {
    float p[6][kBlock];  // scaled position hi (x, y, z), then lo (x, y, z)
    float Rs[kBlock], Rlo[kBlock], inv_m[kBlock];
};

// |pos[B] - pos[A]|^2 in FP64, the formula of the previous-step distance in
// contact_mixed (rare paths: the contact test, write-step energies).
__device__ __forceinline__ double fp64_d2(const System& s, int A, int B)
{
    const double rx = s.pos.c[0][B] - s.pos.c[0][A];
    const double ry = s.pos.c[1][B] - s.pos.c[1][A];
    const double rz = s.pos.c[2][B] - s.pos.c[2][A];
    return fma(rx, rx, fma(ry, ry, rz * rz));
}

// Same tiling as pair_tile_kernel: one warp per lower-triangular 32x32 block
// tile, lane b = sphere 32Y+b, loop over the A block; terms stored as FP32:
// sphere A's in the A-side buffer (the float view of pairbuf), sphere B's in
// the B-side buffer pairT, both at mixed_term_index(A, B): tile (X, Y) of
// both is 4 KB of contiguous memory and each of a warp's stores covers one
// 128-byte row of it.  Torques (contacts only) go to the float view of
// torqbuf, [A][B] and [B][A].
template <bool WRITE>
__global__ void __launch_bounds__(128, 4) mixed_pair_kernel(const __grid_constant__ System s)
{
    __shared__ ABlockMixed sA[4];
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    ABlockMixed& ab = sA[wib];
    const long long nwarps = (long long)gridDim.x * 4;
    const size_t plane = (size_t)s.npad * s.npad;
    float* pbuf = reinterpret_cast<float*>(s.pairbuf);
    float* tbuf = reinterpret_cast<float*>(s.torqbuf);
    const int sh = s.len_shift;
    const float L = ldexpf(1.0f, sh);
    const float hmin_s = (float)s.mat.h_min / L;
    const float c_vdw = (float)(s.mat.Ha / 6 * 64) / L;   // dyn per unit vdw_shape

    for (long long t = (long long)blockIdx.x * 4 + wib; t < s.ntiles; t += nwarps) {
        int X, Y;
        tile_coords(t, X, Y);
        {
            const int i = X * kBlock + lane;
#pragma unroll
            for (int k = 0; k < 6; ++k) ab.p[k][lane] = s.f_pos[k][i];
            ab.Rs[lane] = s.f_R[i]; ab.Rlo[lane] = s.f_Rlo[i]; ab.inv_m[lane] = s.f_inv_m[i];
        }
        __syncwarp();
        const int B = Y * kBlock + lane;
        const bool bvalid = B < s.n;
        float bp[6];
#pragma unroll
        for (int k = 0; k < 6; ++k) bp[k] = s.f_pos[k][B];
        const float Rbs = s.f_R[B], Rblo = s.f_Rlo[B], inv_mb = s.f_inv_m[B];
        const int a_end = min(kBlock, s.n - X * kBlock);
        double pe = 0;
        uint32_t rowbits = 0, colbits = 0;
        // tile (X, Y) of both term buffers; element (a, lane) of row a is at
        // a * 32 + swizzled lane, so a warp's store covers one 128-byte row
        const size_t tile = ((size_t)X * s.nb + Y) * 1024;
        float* tileA = pbuf + tile;
        float* tileT = s.pairT + tile;
        for (int a = 0; a < a_end; ++a) {
            const bool valid = bvalid && (X != Y || lane < a);
            bool contact = false;
            if (valid) {
                const int A = X * kBlock + a;
                // double-float (~48 bits, FP32 pipe): subtraction, |r|^2 and
                // the squared gap g = (R_A + R_B)^2 - |r|^2, in scaled lengths
                const df::F2 rx = df::sub({bp[0], bp[3]}, {ab.p[0][a], ab.p[3][a]});
                const df::F2 ry = df::sub({bp[1], bp[4]}, {ab.p[1][a], ab.p[4][a]});
                const df::F2 rz = df::sub({bp[2], bp[5]}, {ab.p[2][a], ab.p[5][a]});
                const df::F2 d2 = df::add(df::add(df::sqr(rx), df::sqr(ry)), df::sqr(rz));
                const float Ras = ab.Rs[a];
                const df::F2 sum = df::add({Ras, ab.Rlo[a]}, {Rbs, Rblo});
                const df::F2 gap2 = df::sub(df::sqr(sum), d2);
                // FP32 (scaled lengths)
                const float rxs = rx.hi, rys = ry.hi, rzs = rz.hi;
                const float d2s = d2.hi;
                const float inv_d = rsqrtf(d2s);
                const float dist_s = d2s * inv_d;
                const float ovl_s = __fdividef(gap2.hi, Ras + Rbs + dist_s);
                const float nx = rxs * inv_d, ny = rys * inv_d, nz = rzs * inv_d;
                float fx, fy, fz;
                if (gap2.hi > 0.0f || (gap2.hi == 0.0f && gap2.lo > 0.0f)) {
                    contact = true;
                    const ContactIn in = gather_contact(s, A, B);
                    // the kin/kout test compares |r|^2 with the previous step's,
                    // both in FP64 from the FP64 positions with one formula
                    const double d2_64 = fp64_d2(s, A, B);
                    const ContactF o = contact_mixed(in, s.mat, sh, d2_64, nx, ny, nz, dist_s * L, ovl_s * L, Ras,
                                                     Rbs);
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
                    const float h = fmaxf(-ovl_s, hmin_s);                  // :211-215
                    const float f = c_vdw * vdw_shape(h, Ras, Rbs);
                    fx = f * nx; fy = f * ny; fz = f * nz;
                    if (WRITE) {  // write steps only: the FP64 geometry, as the contact branch
                        const double d2_64 = fp64_d2(s, A, B), sum64 = s.R[A] + s.R[B];
                        pe += pair_pe_fp64(s.mat, s.R[A], s.R[B], fma(sum64, sum64, -d2_64), d2_64, false, 0.0);
                    }
                }
                const float ima = ab.inv_m[a];
                const int e = a * 32 + ((((lane >> 2) ^ (a & 7)) << 2) | (lane & 3));  // mixed_term_index
                float* pa = tileA + e;
                __stcs(pa, fx * ima); __stcs(pa + plane, fy * ima); __stcs(pa + 2 * plane, fz * ima);
                float* pb = tileT + e;
                __stcs(pb, -fx * inv_mb); __stcs(pb + plane, -fy * inv_mb); __stcs(pb + 2 * plane, -fz * inv_mb);
            }
            const uint32_t bal = __ballot_sync(0xffffffffu, contact);
            if (lane == a) rowbits = bal;
            if (contact) colbits |= 1u << a;
        }
        if (X == Y) {
            s.cmask[(size_t)(X * kBlock + lane) * s.nb + X] = rowbits | colbits;
        } else {
            s.cmask[(size_t)(X * kBlock + lane) * s.nb + Y] = rowbits;
            s.cmask[(size_t)(Y * kBlock + lane) * s.nb + X] = colbits;
        }
        if (WRITE) {
            for (int off = 16; off > 0; off >>= 1) pe += __shfl_xor_sync(0xffffffffu, pe, off);
            if (lane == 0) s.pe_tile[t] = pe;
        }
        __syncwarp();
    }
}

constexpr int kMixThreads = 32;

// Plain-load form of the row sums (used only when no tensor map could be
// made): thread (c, i) sums the FP32 terms of sphere i in FP64 in ascending
// partner order, torque terms of contact partners likewise, then pass 3.
__global__ void __launch_bounds__(kMixThreads) mixed_rowsum_kernel(const __grid_constant__ System s)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 3 * s.n) return;
    const int c = t / s.n;
    const int i = t - c * s.n;
    const int n = s.n;
    const size_t plane = (size_t)s.npad * s.npad;
    // partners j < i from the A side (i, j), j > i from the B side (j, i)
    const float* pA = reinterpret_cast<const float*>(s.pairbuf) + c * plane;
    const float* pT = s.pairT + c * plane;
    double acc = 0.0;
    for (int j = 0; j < i; ++j) acc += f2d_bits(__ldcs(pA + mixed_term_index(s.nb, i, j)));
    for (int j = i + 1; j < n; ++j) acc += f2d_bits(__ldcs(pT + mixed_term_index(s.nb, j, i)));
    double aacc = 0.0;
    const uint32_t* mrow = s.cmask + (size_t)i * s.nb;
    const float* trow = reinterpret_cast<const float*>(s.torqbuf) + c * plane + (size_t)i * s.npad;
    for (int Y = 0; Y < s.nb; ++Y) {
        uint32_t wd = mrow[Y];
        while (wd) {
            const int b = __ffs(wd) - 1;
            wd &= wd - 1;
            aacc += f2d_bits(trow[Y * kBlock + b]);
        }
    }
    const double dt = s.sc->dt;
    const double v = s.velh.c[c][i] + (.5 * acc) * dt;
    const double wv = s.wh.c[c][i] + (.5 * aacc) * dt;
    s.acc.c[c][i] = acc;
    s.aacc.c[c][i] = aacc;
    s.vel.c[c][i] = v;
    s.w.c[c][i] = wv;
    if (!isfinite(v) || !isfinite(wv) || !isfinite(s.pos.c[c][i])) atomicOr(s.status, 1u);
}

}  // namespace

void launch_step_mixed(const System& s, bool write, int num_sms, cudaStream_t st, StepTimers* tm, bool bulk_rows)
{
    launch_drift(s, st);
    if (tm) cudaEventRecord(tm->ev[0], st);
    long long want = (s.ntiles + 3) / 4;
    long long cap = (long long)num_sms * 4;  // 4 CTAs (16 warps) per SM
    const int pb = (int)(want < cap ? want : cap);
    if (write)
        mixed_pair_kernel<true><<<pb, 128, 0, st>>>(s);
    else
        mixed_pair_kernel<false><<<pb, 128, 0, st>>>(s);
    if (tm) cudaEventRecord(tm->ev[1], st);
    if (bulk_rows)
        launch_rowsum_mixed(s, num_sms, st);
    else
        mixed_rowsum_kernel<<<(3 * s.n + kMixThreads - 1) / kMixThreads, kMixThreads, 0, st>>>(s);
    if (tm) cudaEventRecord(tm->ev[2], st);
    if (write) launch_energy(s, st);
}

}  // namespace sl
