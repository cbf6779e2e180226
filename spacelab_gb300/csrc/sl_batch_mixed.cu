// sl_batch_mixed.cu -- batched solver in the mixed-precision form: the same
// persistent work-queue launch as sl_batch.cu, with the pair pass of the
// mixed form (FP64 displacement, |r|^2 and squared gap; FP32 forces and
// torques; FP64 per-sphere accumulation in ascending partner order; FP64
// write-step potential energy).
#include "sl_batch.h"
#include "sl_batch_common.cuh"
#include "sl_pair_mixed.cuh"

namespace sl {

namespace {

using batch::drift;
using batch::kick;

template <int TILE>
struct JTileM {
    double x[TILE], y[TILE], z[TILE], R[TILE];
    float Rs[TILE];
};

template <int TILE, bool WRITE>
__device__ double pair_pass_mixed(const Batch& b, int off, int n, const Material& M, double kin, double kout,
                                  JTileM<TILE>& jt)
{
    const int sh = b.len_shift;
    const float L = ldexpf(1.0f, sh);
    const float hmin_s = (float)M.h_min / L;
    const float c_vdw = (float)(M.Ha / 6 * 64) / L;
    double pe = 0;
    for (int ibase = 0; ibase < n; ibase += blockDim.x) {
        const int i = ibase + threadIdx.x;
        const bool active = i < n;
        const int gi = off + (active ? i : 0);
        const double xi = b.pos.c[0][gi], yi = b.pos.c[1][gi], zi = b.pos.c[2][gi], Ri = b.R[gi];
        const float Rsi = b.f_R[gi], imi = b.f_inv_m[gi], imoii = b.f_inv_moi[gi];
        double ax = 0, ay = 0, az = 0, tx = 0, ty = 0, tz = 0;
        for (int jbase = 0; jbase < n; jbase += TILE) {
            for (int t = threadIdx.x; t < TILE; t += blockDim.x) {
                const int j = jbase + t;
                if (j < n) {
                    const int g = off + j;
                    jt.x[t] = b.pos.c[0][g]; jt.y[t] = b.pos.c[1][g]; jt.z[t] = b.pos.c[2][g];
                    jt.R[t] = b.R[g]; jt.Rs[t] = b.f_R[g];
                }
            }
            __syncthreads();
            if (active) {
                const int jend = min(TILE, n - jbase);
                for (int t = 0; t < jend; ++t) {
                    const int j = jbase + t;
                    if (j == i) continue;
                    const bool iA = i > j;
                    // r = pos[B] - pos[A] in FP64; the sign flips with the orientation
                    const double rx = iA ? jt.x[t] - xi : xi - jt.x[t];
                    const double ry = iA ? jt.y[t] - yi : yi - jt.y[t];
                    const double rz = iA ? jt.z[t] - zi : zi - jt.z[t];
                    const double d2 = fma(rx, rx, fma(ry, ry, rz * rz));
                    const double RA = iA ? Ri : jt.R[t], RB = iA ? jt.R[t] : Ri;
                    const double sum = RA + RB;
                    const double gap2 = fma(sum, sum, -d2);
                    const float Ras = iA ? Rsi : jt.Rs[t], Rbs = iA ? jt.Rs[t] : Rsi;
                    const float rxs = d2f_bits(rx, sh), rys = d2f_bits(ry, sh), rzs = d2f_bits(rz, sh);
                    const float d2s = d2f_bits(d2, 2 * sh);
                    const float inv_d = rsqrtf(d2s);
                    const float dist_s = d2s * inv_d;
                    const float ovl_s = __fdividef(d2f_bits(gap2, 2 * sh), Ras + Rbs + dist_s);
                    const float nx = rxs * inv_d, ny = rys * inv_d, nz = rzs * inv_d;
                    float fx, fy, fz;
                    if (gap2 > 0.0) {
                        const int gA = off + (iA ? i : j), gB = off + (iA ? j : i);
                        ContactIn in;
                        for (int c = 0; c < 3; ++c) {
                            in.prevA[c] = b.prev.c[c][gA]; in.prevB[c] = b.prev.c[c][gB];
                            in.wA[c] = b.w.c[c][gA]; in.wB[c] = b.w.c[c][gB];
                            in.vA[c] = b.vel.c[c][gA]; in.vB[c] = b.vel.c[c][gB];
                        }
                        in.mA = b.m[gA]; in.mB = b.m[gB]; in.kin = kin; in.kout = kout;
                        const ContactF o = contact_mixed(in, M, sh, d2, nx, ny, nz, dist_s * L, ovl_s * L, Ras, Rbs);
                        fx = o.fx; fy = o.fy; fz = o.fz;
                        const float qx = iA ? o.tax : o.tbx, qy = iA ? o.tay : o.tby, qz = iA ? o.taz : o.tbz;
                        tx += f2d_bits(qx * imoii); ty += f2d_bits(qy * imoii); tz += f2d_bits(qz * imoii);
                        if (WRITE && iA) pe += pair_pe_fp64(M, RA, RB, gap2, d2, true, o.k);
                    } else {
                        const float h = fmaxf(-ovl_s, hmin_s);
                        const float f = c_vdw * vdw_shape(h, Ras, Rbs);
                        fx = f * nx; fy = f * ny; fz = f * nz;
                        if (WRITE && iA) pe += pair_pe_fp64(M, RA, RB, gap2, d2, false, 0.0);
                    }
                    const float s = iA ? imi : -imi;  // acc[A] += F/m[A]; acc[B] -= F/m[B]
                    ax += f2d_bits(fx * s); ay += f2d_bits(fy * s); az += f2d_bits(fz * s);
                }
            }
            __syncthreads();
        }
        if (active) {
            b.acc.c[0][gi] = ax; b.acc.c[1][gi] = ay; b.acc.c[2][gi] = az;
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
