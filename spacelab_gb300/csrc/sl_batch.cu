// sl_batch.cu -- batched exact FP64 solver: thousands of independent
// systems (projectile-target collisions of uneven sphere counts) advanced by
// ONE persistent launch.
//
// Each CTA takes whole instances from an atomic work queue (largest first)
// and runs all of an instance's steps before taking the next one; the only
// synchronisation is __syncthreads inside the CTA, so no CTA ever waits on
// another.  Within an instance a step is the reference's three passes
// (ColliderSingleCore.cpp:82-97, 100-256, 263-287):
//   drift    one thread per sphere (strided);
//   pairs    either the pair-tile pass (shape tile 0: every pair once into
//            the CTA's pair-term buffers by the single system's tile routine,
//            then ordered row sums), or the per-sphere loop: thread i walks
//            partners j ascending through j-tiles staged in shared memory and
//            adds each term to its running sum in the order the reference
//            adds them to acc[i].  Either way the result is bit-identical to
//            the reference step, pair terms being computed in the
//            reference's (A = max, B = min) orientation;
//   kick     pass 3, plus the write-step energy totals reduced in a fixed
//            tree inside the CTA.
// The pass, its j-tile size and the threads per instance (block size) are
// chosen by the host autotuner (sl_batch_capi.cu).
#include "sl_batch.h"
#include "sl_batch_common.cuh"
#include "sl_fp64_exact.cuh"
#include "sl_pair_exact.cuh"
#include "sl_tile_exact.cuh"
#include "sl_vdw_energy.cuh"

namespace sl {

namespace {

using batch::cta_sum8;
using batch::drift;
using batch::kick;

template <int TILE>
struct JTile {
    double x[TILE], y[TILE], z[TILE], R[TILE], twoR[TILE], fourR[TILE], cR3[TILE];
};

// Pass 2 for one instance; returns this thread's share of the PE (pairs
// are counted once, by the thread of sphere A).
template <int TILE, bool WRITE>
__device__ double pair_pass(const Batch& b, int off, int n, const Material& M, double kin, double kout,
                            JTile<TILE>& jt)
{
    double pe = 0;
    for (int ibase = 0; ibase < n; ibase += blockDim.x) {
        const int i = ibase + threadIdx.x;
        const bool active = i < n;
        const int gi = off + (active ? i : 0);
        const double xi = b.pos.c[0][gi], yi = b.pos.c[1][gi], zi = b.pos.c[2][gi];
        const double Ri = b.R[gi], twoRi = b.twoR[gi], fourRi = b.fourR[gi], cR3i = b.cR3[gi];
        const double mi = b.m[gi], moii = b.moi[gi], imoii = b.inv_moi[gi];
        const unsigned long long rmi = b.rm[gi];
        double ax = 0, ay = 0, az = 0, tx = 0, ty = 0, tz = 0;
        for (int jbase = 0; jbase < n; jbase += TILE) {
            for (int t = threadIdx.x; t < TILE; t += blockDim.x) {
                const int j = jbase + t;
                if (j < n) {
                    const int g = off + j;
                    jt.x[t] = b.pos.c[0][g]; jt.y[t] = b.pos.c[1][g]; jt.z[t] = b.pos.c[2][g];
                    jt.R[t] = b.R[g]; jt.twoR[t] = b.twoR[g]; jt.fourR[t] = b.fourR[g]; jt.cR3[t] = b.cR3[g];
                }
            }
            __syncthreads();
            if (active) {
                const int jend = min(TILE, n - jbase);
                for (int t = 0; t < jend; ++t) {
                    const int j = jbase + t;
                    if (j == i) continue;
                    const bool iA = i > j;  // the reference's orientation: A = max, B = min
                    const double Ax = iA ? xi : jt.x[t], Ay = iA ? yi : jt.y[t], Az = iA ? zi : jt.z[t];
                    const double Bx = iA ? jt.x[t] : xi, By = iA ? jt.y[t] : yi, Bz = iA ? jt.z[t] : zi;
                    const double RA = iA ? Ri : jt.R[t], RB = iA ? jt.R[t] : Ri;
                    const double twoRA = iA ? twoRi : jt.twoR[t], twoRB = iA ? jt.twoR[t] : twoRi;
                    const double fourRA = iA ? fourRi : jt.fourR[t], cR3A = iA ? cR3i : jt.cR3[t];
                    const double sumRaRb = RA + RB;                                  // :104
                    const double rx = Bx - Ax, ry = By - Ay, rz = Bz - Az;           // :105
                    const double d2 = rx * rx + ry * ry + rz * rz;
                    int p;
                    unsigned long long F;
                    const unsigned long long Y = rsqrt_fix(d2, p, F);
                    const double dist = sqrt_fix(d2, F, Y, p);                       // :107
                    const double overlap = sumRaRb - dist;                           // :110
                    double fx, fy, fz;
                    if (overlap > 0) {
                        const int gA = off + (iA ? i : j), gB = off + (iA ? j : i);
                        ContactIn in;
                        for (int c = 0; c < 3; ++c) {
                            in.prevA[c] = b.prev.c[c][gA]; in.prevB[c] = b.prev.c[c][gB];
                            in.wA[c] = b.w.c[c][gA]; in.wB[c] = b.w.c[c][gB];
                            in.vA[c] = b.vel.c[c][gA]; in.vB[c] = b.vel.c[c][gB];
                        }
                        in.mA = b.m[gA]; in.mB = b.m[gB]; in.kin = kin; in.kout = kout;
                        const ContactOut o = contact_pair_exact<WRITE>(in, M, rx, ry, rz, dist, overlap, RA, RB,
                                                                       twoRA, twoRB, fourRA, cR3A);
                        fx = o.fx; fy = o.fy; fz = o.fz;
                        const double qx = iA ? o.tax : o.tbx, qy = iA ? o.tay : o.tby, qz = iA ? o.taz : o.tbz;
                        tx += div_by_recip(qx, moii, imoii);                         // :187-188
                        ty += div_by_recip(qy, moii, imoii);
                        tz += div_by_recip(qz, moii, imoii);
                        if (WRITE && iA) pe += o.pe;
                    } else {
                        double h = fabs(overlap);                                    // :211-215
                        if (h < M.h_min) h = M.h_min;
                        const double coef = vdw_coef_fix(h, RA, RB, twoRA, twoRB, fourRA, cR3A);
                        fx = coef * div_by_rsqrt(rx, dist, Y, p);
                        fy = coef * div_by_rsqrt(ry, dist, Y, p);
                        fz = coef * div_by_rsqrt(rz, dist, Y, p);
                        if (WRITE && iA) pe += vdw_energy_far_df(M.Ha, h, RA, RB, twoRA);
                    }
                    const double qx = div_by_fixed<false>(fx, mi, rmi);              // :249-250
                    const double qy = div_by_fixed<false>(fy, mi, rmi);
                    const double qz = div_by_fixed<false>(fz, mi, rmi);
                    if (iA) { ax += qx; ay += qy; az += qz; }
                    else { ax -= qx; ay -= qy; az -= qz; }
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
__global__ void __launch_bounds__(256) batch_exact_kernel(const __grid_constant__ Batch b, int first_step, int nsteps,
                                                          int skip, int do_init)
{
    __shared__ JTile<TILE> jt;
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
        if (do_init) {  // initial forces: a step with dt = 0 (init_conditions)
            drift(b, off, n, 0.0);
            __syncthreads();
            const double pe = pair_pass<TILE, true>(b, off, n, M, kin, kout, jt);
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
                pe = pair_pass<TILE, true>(b, off, n, M, kin, kout, jt);
            else
                pair_pass<TILE, false>(b, off, n, M, kin, kout, jt);
            __syncthreads();
            const int r = write ? step / skip : 0;
            kick(b, inst, off, n, dt, write, pe, recs + (size_t)(r < b.nrec ? r : b.nrec - 1) * 8, sh);
            __syncthreads();
        }
    }
}

// ---------------------------------------------------------------------------
// Pair-tile pass (shape tile 0): every pair once, as the single-system step
// does it.  The CTA's warps take the instance's 32 x 32 block tiles and run
// the single system's tile routine (tile_pairs, sl_tile_exact.cuh) on a
// System view of the instance whose pair-term, torque and contact buffers are
// the CTA's scratch; then thread (c, i) adds row i of the pair terms in
// ascending partner order and its contact torques likewise -- the
// reference's order, so the result stays bit-identical -- and the half-kick
// follows.  This evaluates each pair once where the per-sphere loop does it
// twice, at the price of the row sums' dependent FP64 adds.
__device__ void make_view(System& v, const Batch& b, int inst, int off, int n)
{
    v = System{};
    v.n = n;
    v.nb = (n + kBlock - 1) / kBlock;
    v.npad = b.x_np;  // the scratch's row stride
    v.ntiles = (long long)v.nb * (v.nb + 1) / 2;
    v.nitems = v.ntiles;
    const Vec3Soa* src[8] = {&b.pos, &b.prev, &b.vel, &b.velh, &b.w, &b.wh, &b.acc, &b.aacc};
    Vec3Soa* dst[8] = {&v.pos, &v.prev, &v.vel, &v.velh, &v.w, &v.wh, &v.acc, &v.aacc};
    for (int k = 0; k < 8; ++k)
        for (int c = 0; c < 3; ++c) dst[k]->c[c] = src[k]->c[c] + off;
    v.R = b.R + off; v.m = b.m + off; v.moi = b.moi + off;
    v.twoR = b.twoR + off; v.fourR = b.fourR + off; v.cR3 = b.cR3 + off;
    v.rm = b.rm + off; v.inv_moi = b.inv_moi + off;
    v.pairbuf = b.xpair + (size_t)blockIdx.x * b.xpair_cta;
    v.torqbuf = b.xtorq + (size_t)blockIdx.x * b.xpair_cta;
    v.cmask = b.xmask + (size_t)blockIdx.x * b.xmask_cta;
    v.sc = b.isc + inst;
    v.mat = b.mat;
    v.mat.u_s = b.u_s[inst];
}

template <bool WRITE>
__device__ double exact_tile_pass(const System& s, ABlock* blocks)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    ABlock& ab = blocks[warp];
    const int n = s.n;
    const double Ha = s.mat.Ha;
    const long long h_min_bits = __double_as_longlong(s.mat.h_min);  // h_min > 0
    double pe = 0;
    for (long long t = warp; t < s.ntiles; t += nwarps) {
        int X, Y;
        tile_coords(t, X, Y);
        {
            const int i = min(X * kBlock + lane, n - 1);  // padding rows repeat the last sphere (never paired)
            ab.x[lane] = s.pos.c[0][i]; ab.y[lane] = s.pos.c[1][i]; ab.z[lane] = s.pos.c[2][i];
            ab.R[lane] = s.R[i]; ab.twoR[lane] = s.twoR[i]; ab.fourR[lane] = s.fourR[i];
            ab.cR3[lane] = s.cR3[i]; ab.m[lane] = s.m[i]; ab.rm[lane] = s.rm[i];
        }
        __syncwarp();
        const int B = Y * kBlock + lane;
        const bool bvalid = B < n;
        const int Bc = min(B, n - 1);
        const double bx = s.pos.c[0][Bc], by = s.pos.c[1][Bc], bz = s.pos.c[2][Bc];
        const double Rb = s.R[Bc], twoRb = s.twoR[Bc], mb = s.m[Bc];
        const unsigned long long rmb = s.rm[Bc];
        const double R0 = ab.R[0];
        const bool uni = __all_sync(0xffffffffu, ab.R[lane] == R0 && Rb == R0);
        const double twoR0 = ab.twoR[0], sum0 = R0 + R0, c40 = ab.fourR[0] * R0;
        const double P0 = ab.cR3[0] * R0 * R0 * R0;
        const int a_end = min(kBlock, n - X * kBlock);
        uint32_t rowbits = 0, colbits = 0;
        double* rowA = s.pairbuf + (size_t)(X * kBlock) * s.npad + B;  // + a*npad: term for A
        double* rowB = s.pairbuf + (size_t)B * s.npad + X * kBlock;    // + a: term for B
        const TileUniform tu{R0, twoR0, sum0, c40, P0};
        if (uni)
            tile_pairs<WRITE, true>(s, ab, X, Y, lane, a_end, bx, by, bz, Rb, twoRb, mb, rmb, bvalid, tu, h_min_bits,
                                    Ha, rowA, rowB, pe, rowbits, colbits);
        else
            tile_pairs<WRITE, false>(s, ab, X, Y, lane, a_end, bx, by, bz, Rb, twoRb, mb, rmb, bvalid, tu, h_min_bits,
                                     Ha, rowA, rowB, pe, rowbits, colbits);
        if (X == Y) {
            s.cmask[(size_t)(X * kBlock + lane) * s.nb + X] = rowbits | colbits;
        } else {
            s.cmask[(size_t)(X * kBlock + lane) * s.nb + Y] = rowbits;
            s.cmask[(size_t)(Y * kBlock + lane) * s.nb + X] = colbits;
        }
        __syncwarp();
    }
    return pe;
}

// Thread (c, i): acc_c[i] and aacc_c[i] in the reference's order
// (ColliderSingleCore.cpp:100-103, 249-250): partners j < i, then j > i.
__device__ void exact_row_sums(const System& s)
{
    const int n = s.n;
    const size_t plane = (size_t)s.npad * s.npad;
    for (int t = threadIdx.x; t < 3 * n; t += blockDim.x) {
        const int c = t / n, i = t - c * n;
        const double* row = s.pairbuf + c * plane + (size_t)i * s.npad;
        double acc = 0;
        for (int j = 0; j < i; ++j) acc += row[j];
        for (int j = i + 1; j < n; ++j) acc += row[j];
        const double* trow = s.torqbuf + c * plane + (size_t)i * s.npad;
        const uint32_t* mrow = s.cmask + (size_t)i * s.nb;
        double aacc = 0;
        for (int Y = 0; Y < s.nb; ++Y) {
            uint32_t wd = mrow[Y];
            while (wd) {
                const int j = Y * kBlock + __ffs(wd) - 1;
                wd &= wd - 1;
                aacc += trow[j];
            }
        }
        s.acc.c[c][i] = acc;
        s.aacc.c[c][i] = aacc;
    }
}

constexpr int kExactTileWarps = 8;

__global__ void __launch_bounds__(32 * kExactTileWarps) batch_exact_tiles_kernel(const __grid_constant__ Batch b,
                                                                                int first_step, int nsteps, int skip,
                                                                                int do_init)
{
    __shared__ ABlock blocks[kExactTileWarps];
    __shared__ System sv;
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
        const double dt = b.dt[inst];
        double* recs = b.energy + (size_t)inst * b.nrec * 8;
        if (threadIdx.x == 0) make_view(sv, b, inst, off, n);
        __syncthreads();
        if (do_init) {
            drift(b, off, n, 0.0);
            __syncthreads();
            const double pe = exact_tile_pass<true>(sv, blocks);
            __syncthreads();
            exact_row_sums(sv);
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
                pe = exact_tile_pass<true>(sv, blocks);
            else
                exact_tile_pass<false>(sv, blocks);
            __syncthreads();
            exact_row_sums(sv);
            __syncthreads();
            const int r = write ? step / skip : 0;
            kick(b, inst, off, n, dt, write, pe, recs + (size_t)(r < b.nrec ? r : b.nrec - 1) * 8, sh);
            __syncthreads();
        }
    }
}

__global__ void batch_derive_kernel(const __grid_constant__ Batch b)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= b.total) return;
    const double R = b.R[i], m = b.m[i], moi = b.moi[i];
    b.twoR[i] = 2 * R;
    b.fourR[i] = 4 * R;
    b.cR3[i] = b.mat.Ha / 6 * 64 * R * R * R;
    b.rm[i] = recip_of(m);
    b.inv_moi[i] = 1.0 / moi;
    if (b.f_R) {  // mixed form: slot i holds sphere perm[i]
        const int g = b.perm[i];
        const double Rg = b.R[g];
        const float rh = d2f_bits(Rg, b.len_shift);
        b.f_R[i] = rh;
        b.f_Rlo[i] = d2f_bits(Rg - f2d_bits(rh) * ldexp(1.0, b.len_shift), b.len_shift);
        b.f_inv_m[i] = d2f_bits(1.0 / b.m[g], 0);
        b.f_inv_moi[i] = d2f_bits(1.0 / b.moi[g], 0);
    }
}

}  // namespace

void launch_batch_derive(const Batch& b, cudaStream_t st)
{
    batch_derive_kernel<<<(b.total + 255) / 256, 256, 0, st>>>(b);
}

void launch_batch_exact(const Batch& b, int tile, int threads, int blocks, int first_step, int nsteps, int skip,
                        int do_init, cudaStream_t st)
{
    switch (tile) {
        case 0: batch_exact_tiles_kernel<<<blocks, threads, 0, st>>>(b, first_step, nsteps, skip, do_init); break;
        case 32: batch_exact_kernel<32><<<blocks, threads, 0, st>>>(b, first_step, nsteps, skip, do_init); break;
        case 64: batch_exact_kernel<64><<<blocks, threads, 0, st>>>(b, first_step, nsteps, skip, do_init); break;
        default: batch_exact_kernel<128><<<blocks, threads, 0, st>>>(b, first_step, nsteps, skip, do_init); break;
    }
}

int batch_max_blocks_per_sm(int tile, int threads, bool mixed)
{
    if (mixed) return batch_mixed_max_blocks_per_sm(tile, threads);
    int nb = 0;
    switch (tile) {
        case 0: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, batch_exact_tiles_kernel, threads, 0); break;
        case 32: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, batch_exact_kernel<32>, threads, 0); break;
        case 64: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, batch_exact_kernel<64>, threads, 0); break;
        default: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, batch_exact_kernel<128>, threads, 0); break;
    }
    return nb;
}

}  // namespace sl
