// sl_batch_mixed.cu -- batched solver in the mixed-precision form: the same
// persistent work-queue launch as sl_batch.cu, with the pair pass of the
// mixed form: double-float (sl_df.cuh) displacement, |r|^2 and squared gap
// from double-float splits of the scaled positions; FP32 forces and torques;
// compensated FP32 per-sphere sums in ascending partner order, converted to
// FP64; FP64 kin/kout test and write-step potential energy from the FP64
// positions.  The non-contact pair path issues no FP64 instruction.
#include "sl_batch.h"
#include "sl_batch_common.cuh"
#include "sl_df.cuh"
#include "sl_pair_mixed.cuh"

namespace sl {

namespace {

using batch::drift;
using batch::kick;

template <int TILE>
struct JTileM {
    float ph[3][TILE], pl[3][TILE];  // scaled position, double-float hi and lo
    float Rs[TILE], Rlo[TILE];       // scaled radius, double-float hi and lo
};

// x * 2^-sh as a double-float (hi, lo)
__device__ __forceinline__ df::F2 split_scaled(double x, int sh, double scale)
{
    const float hi = d2f_bits(x, sh);
    return {hi, d2f_bits(x - f2d_bits(hi) * scale, sh)};
}

// |pos[gB] - pos[gA]|^2 in FP64, the previous-step formula of contact_mixed
__device__ __forceinline__ double fp64_d2(const Batch& b, int gA, int gB)
{
    const double rx = b.pos.c[0][gB] - b.pos.c[0][gA];
    const double ry = b.pos.c[1][gB] - b.pos.c[1][gA];
    const double rz = b.pos.c[2][gB] - b.pos.c[2][gA];
    return fma(rx, rx, fma(ry, ry, rz * rz));
}

template <int TILE, bool WRITE>
__device__ double pair_pass_mixed(const Batch& b, int off, int n, const Material& M, double kin, double kout,
                                  JTileM<TILE>& jt)
{
    const int sh = b.len_shift;
    const float L = ldexpf(1.0f, sh);
    const float hmin_s = (float)M.h_min / L;
    const float c_vdw = (float)(M.Ha / 6 * 64) / L;
    const double scale = ldexp(1.0, sh);
    double pe = 0;
    for (int ibase = 0; ibase < n; ibase += blockDim.x) {
        const int i = ibase + threadIdx.x;
        const bool active = i < n;
        const int gi = off + (active ? i : 0);
        df::F2 pi[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) pi[c] = split_scaled(b.pos.c[c][gi], sh, scale);
        const df::F2 Ri = split_scaled(b.R[gi], sh, scale);
        const float imi = b.f_inv_m[gi], imoii = b.f_inv_moi[gi];
        df::Sum ax{0.0f, 0.0f}, ay{0.0f, 0.0f}, az{0.0f, 0.0f};
        double tx = 0, ty = 0, tz = 0;
        for (int jbase = 0; jbase < n; jbase += TILE) {
            for (int t = threadIdx.x; t < TILE; t += blockDim.x) {
                const int j = jbase + t;
                if (j < n) {
                    const int g = off + j;
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        const df::F2 v = split_scaled(b.pos.c[c][g], sh, scale);
                        jt.ph[c][t] = v.hi;
                        jt.pl[c][t] = v.lo;
                    }
                    const df::F2 r = split_scaled(b.R[g], sh, scale);
                    jt.Rs[t] = r.hi;
                    jt.Rlo[t] = r.lo;
                }
            }
            __syncthreads();
            if (active) {
                const int jend = min(TILE, n - jbase);
                for (int t = 0; t < jend; ++t) {
                    const int j = jbase + t;
                    if (j == i) continue;
                    const bool iA = i > j;
                    // r = pos[B] - pos[A] in double-float; the sign flips with the orientation
                    df::F2 r3[3];
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        const df::F2 pj{jt.ph[c][t], jt.pl[c][t]};
                        r3[c] = iA ? df::sub(pj, pi[c]) : df::sub(pi[c], pj);
                    }
                    const df::F2 d2 = df::add(df::add(df::sqr(r3[0]), df::sqr(r3[1])), df::sqr(r3[2]));
                    const df::F2 sum = df::add(Ri, {jt.Rs[t], jt.Rlo[t]});
                    const df::F2 gap2 = df::sub(df::sqr(sum), d2);
                    const float Ras = iA ? Ri.hi : jt.Rs[t], Rbs = iA ? jt.Rs[t] : Ri.hi;
                    const float rxs = r3[0].hi, rys = r3[1].hi, rzs = r3[2].hi;
                    const float d2s = d2.hi;
                    const float inv_d = rsqrtf(d2s);
                    const float dist_s = d2s * inv_d;
                    const float ovl_s = __fdividef(gap2.hi, Ras + Rbs + dist_s);
                    const float nx = rxs * inv_d, ny = rys * inv_d, nz = rzs * inv_d;
                    float fx, fy, fz;
                    const int gA = off + (iA ? i : j), gB = off + (iA ? j : i);
                    if (gap2.hi > 0.0f || (gap2.hi == 0.0f && gap2.lo > 0.0f)) {
                        ContactIn in;
                        for (int c = 0; c < 3; ++c) {
                            in.prevA[c] = b.prev.c[c][gA]; in.prevB[c] = b.prev.c[c][gB];
                            in.wA[c] = b.w.c[c][gA]; in.wB[c] = b.w.c[c][gB];
                            in.vA[c] = b.vel.c[c][gA]; in.vB[c] = b.vel.c[c][gB];
                        }
                        in.mA = b.m[gA]; in.mB = b.m[gB]; in.kin = kin; in.kout = kout;
                        // kin/kout: |r|^2 against the previous step's, both FP64 by one formula
                        const double d2_64 = fp64_d2(b, gA, gB);
                        const ContactF o = contact_mixed(in, M, sh, d2_64, nx, ny, nz, dist_s * L, ovl_s * L, Ras,
                                                         Rbs);
                        fx = o.fx; fy = o.fy; fz = o.fz;
                        const float qx = iA ? o.tax : o.tbx, qy = iA ? o.tay : o.tby, qz = iA ? o.taz : o.tbz;
                        tx += f2d_bits(qx * imoii); ty += f2d_bits(qy * imoii); tz += f2d_bits(qz * imoii);
                        if (WRITE && iA) {
                            const double sum64 = b.R[gA] + b.R[gB];
                            pe += pair_pe_fp64(M, b.R[gA], b.R[gB], fma(sum64, sum64, -d2_64), d2_64, true, o.k);
                        }
                    } else {
                        const float h = fmaxf(-ovl_s, hmin_s);
                        const float f = c_vdw * vdw_shape(h, Ras, Rbs);
                        fx = f * nx; fy = f * ny; fz = f * nz;
                        if (WRITE && iA) {
                            const double d2_64 = fp64_d2(b, gA, gB), sum64 = b.R[gA] + b.R[gB];
                            pe += pair_pe_fp64(M, b.R[gA], b.R[gB], fma(sum64, sum64, -d2_64), d2_64, false, 0.0);
                        }
                    }
                    const float s = iA ? imi : -imi;  // acc[A] += F/m[A]; acc[B] -= F/m[B]
                    ax.add(fx * s); ay.add(fy * s); az.add(fz * s);
                }
            }
            __syncthreads();
        }
        if (active) {
            b.acc.c[0][gi] = f2d_bits(ax.s) + f2d_bits(ax.c);
            b.acc.c[1][gi] = f2d_bits(ay.s) + f2d_bits(ay.c);
            b.acc.c[2][gi] = f2d_bits(az.s) + f2d_bits(az.c);
            b.aacc.c[0][gi] = tx; b.aacc.c[1][gi] = ty; b.aacc.c[2][gi] = tz;
        }
    }
    return pe;
}

template <int TILE>
__global__ void __launch_bounds__(256) batch_mixed_kernel(const __grid_constant__ Batch b, int first_step, int nsteps,
                                                          int skip, int do_init)
{
    __shared__ JTileM<TILE> jt;
    __shared__ double sh[8][32];
    __shared__ int s_next;
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) s_next = atomicAdd(b.counter, 1);
        __syncthreads();
        const int k = s_next;
        if (k >= b.ninst) return;
        const int inst = b.order[k];
        const int off = b.off[inst], n = b.cnt[inst];
        Material M = b.mat;
        M.u_s = b.u_s[inst];
        const double dt = b.dt[inst], kin = b.kin[inst], kout = b.kout[inst];
        double* recs = b.energy + (size_t)inst * b.nrec * 8;
        if (do_init) {
            drift(b, off, n, 0.0);
            __syncthreads();
            const double pe = pair_pass_mixed<TILE, true>(b, off, n, M, kin, kout, jt);
            __syncthreads();
            kick(b, inst, off, n, 0.0, true, pe, recs, sh);
            __syncthreads();
        }
        for (int q = 0; q < nsteps; ++q) {
            const int step = first_step + q;
            const bool write = skip > 0 && step % skip == 0;
            drift(b, off, n, dt);
            __syncthreads();
            double pe = 0;
            if (write)
                pe = pair_pass_mixed<TILE, true>(b, off, n, M, kin, kout, jt);
            else
                pair_pass_mixed<TILE, false>(b, off, n, M, kin, kout, jt);
            __syncthreads();
            const int r = write ? step / skip : 0;
            kick(b, inst, off, n, dt, write, pe, recs + (size_t)(r < b.nrec ? r : b.nrec - 1) * 8, sh);
            __syncthreads();
        }
    }
}

}  // namespace

void launch_batch_mixed(const Batch& b, int tile, int threads, int blocks, int first_step, int nsteps, int skip,
                        int do_init, cudaStream_t st)
{
    switch (tile) {
        case 32: batch_mixed_kernel<32><<<blocks, threads, 0, st>>>(b, first_step, nsteps, skip, do_init); break;
        case 64: batch_mixed_kernel<64><<<blocks, threads, 0, st>>>(b, first_step, nsteps, skip, do_init); break;
        default: batch_mixed_kernel<128><<<blocks, threads, 0, st>>>(b, first_step, nsteps, skip, do_init); break;
    }
}

int batch_mixed_max_blocks_per_sm(int tile, int threads)
{
    int nb = 0;
    switch (tile) {
        case 32: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, batch_mixed_kernel<32>, threads, 0); break;
        case 64: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, batch_mixed_kernel<64>, threads, 0); break;
        default: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, batch_mixed_kernel<128>, threads, 0); break;
    }
    return nb;
}

}  // namespace sl
