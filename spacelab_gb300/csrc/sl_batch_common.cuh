// sl_batch_common.cuh -- per-instance passes 1 and 3 of the batched solver
// (ColliderSingleCore.cpp:82-97, 263-287) and the CTA reduction of the
// energy totals, shared by the exact and mixed batched kernels.  Each
// function is executed by all threads of a CTA for one instance.
#pragma once
#include "sl_batch.h"

namespace sl {
namespace batch {

// Deterministic CTA sum of 8 values per thread; result valid in thread 0.
__device__ __forceinline__ void cta_sum8(double v[8], double (*sh)[32])
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int k = 0; k < 8; ++k)
        for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
    if (lane == 0)
        for (int k = 0; k < 8; ++k) sh[k][warp] = v[k];
    __syncthreads();
    if (threadIdx.x == 0)
        for (int k = 0; k < 8; ++k) {
            double s = 0;
            for (int q = 0; q < nw; ++q) s += sh[k][q];
            v[k] = s;
        }
    __syncthreads();
}

__device__ __forceinline__ void drift(const Batch& b, int off, int n, double dt)
{
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int g = b.perm ? b.perm[off + i] : off + i;  // the mixed form walks slots (sl_batch.h)
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const double vh = b.vel.c[c][g] + (.5 * b.acc.c[c][g]) * dt;   // :84
            const double whc = b.w.c[c][g] + (.5 * b.aacc.c[c][g]) * dt;   // :87
            const double p = b.pos.c[c][g];
            b.velh.c[c][g] = vh;
            b.wh.c[c][g] = whc;
            b.prev.c[c][g] = p;
            b.pos.c[c][g] = p + vh * dt;                                   // :90
        }
        if (b.f_pos[0]) {  // mixed form: scaled positions as double-float hi + lo, in slot off + i
            const double scale = ldexp(1.0, b.len_shift);
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const double p = b.pos.c[c][g];
                const float hi = d2f_bits(p, b.len_shift);
                b.f_pos[c][off + i] = hi;
                b.f_pos[3 + c][off + i] = d2f_bits(p - f2d_bits(hi) * scale, b.len_shift);
            }
        }
    }
}

// Pass 3 and, on write steps, the energy record of this instance.
__device__ __forceinline__ void kick(const Batch& b, int inst, int off, int n, double dt, bool write, double pe, double* rec,
                     double (*sh)[32])
{
    double e[8] = {pe, 0, 0, 0, 0, 0, 0, 0};
    bool bad = false;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int g = off + i;
        double v[3], w[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            v[c] = b.velh.c[c][g] + (.5 * b.acc.c[c][g]) * dt;    // :265
            w[c] = b.wh.c[c][g] + (.5 * b.aacc.c[c][g]) * dt;     // :266
            b.vel.c[c][g] = v[c];
            b.w.c[c][g] = w[c];
            bad |= !isfinite(v[c]) || !isfinite(w[c]) || !isfinite(b.pos.c[c][g]);
        }
        if (write) {
            const double m = b.m[g], moi = b.moi[g];
            const double px = b.pos.c[0][g], py = b.pos.c[1][g], pz = b.pos.c[2][g];
            e[1] += .5 * m * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]) + .5 * moi * (w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
            e[2] += m * v[0]; e[3] += m * v[1]; e[4] += m * v[2];
            e[5] += m * (py * v[2] - pz * v[1]) + moi * w[0];
            e[6] += m * (pz * v[0] - px * v[2]) + moi * w[1];
            e[7] += m * (px * v[1] - py * v[0]) + moi * w[2];
        }
    }
    if (bad) atomicOr(&b.status[inst], 1u);
    if (write) {
        cta_sum8(e, sh);
        if (threadIdx.x == 0)
            for (int k = 0; k < 8; ++k) rec[k] = e[k];
    }
}

}  // namespace batch
}  // namespace sl
