// sl_step.cu -- the FP64 step of SpaceLab's hot path on sm_103a, bit-exact
// with the reference's sim_one_step (ColliderSingleCore.cpp:78-288).
//
// One step is four launches on the handle's stream (the row sums have a
// TMA-streamed form in sl_rowsum_tma.cu, used whenever a tensor map of the
// pair-term buffer could be made):
//   drift_kernel      pass 1 (ColliderSingleCore.cpp:82-97): velh, wh, drift,
//                     and the previous positions that replace the reference's
//                     O(N^2) `distances` array (ball_group.hpp:741).
//   pair_tile_kernel  pass 2 (:100-256): every unordered pair (A > B) is
//                     evaluated ONCE, in the reference's orientation, by one
//                     lane of a warp that owns a 32x32 block tile; its terms
//                     for both spheres go to pairbuf/torqbuf.
//   rowsum_kernel     sums row s of pairbuf in ascending partner order -- the
//                     order in which the reference adds terms to acc[s] --
//                     then pass 3 (:263-267): vel, w.
//   energy kernels    write steps only: PE from per-tile partials, KE, |p|,
//                     |L| (:282-285), in a fixed reduction tree.
// All arithmetic follows the reference's vec3 evaluation order
// (vec3.hpp:44-128,180-184) and this file is compiled with --fmad=false, so
// no multiply-add is contracted.  The square root and the quotients of the
// non-contact path and of the mass divisions are formed as FP64 estimates
// rounded exactly with integer arithmetic (sl_fp64_exact.cuh): the same
// IEEE results with most of the work moved off the narrow FP64 pipe.  The
// estimates themselves come from the integer pipe too: fixed-point mass
// reciprocals made once at upload, a fixed-point 1/sqrt(d2) by Newton
// iteration, and a fixed-point reciprocal of the vdW denominator.
#include "sl_device.cuh"
#include "sl_kernels.h"
#include "sl_fp64_exact.cuh"
#include "sl_pair_exact.cuh"
#include "sl_tile_exact.cuh"

#include <cstdio>

namespace sl {

// ---------------------------------------------------------------- pass 1 --
// One thread per (component, sphere), in small blocks: the few FP64
// operations per thread then spread over every SM sub-partition's FP64 unit
// (one warp instruction per ~64 cycles each) instead of queueing on a few.
constexpr int kDriftThreads = 64;

__global__ void __launch_bounds__(kDriftThreads) drift_kernel(const __grid_constant__ System s)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 3 * s.n) return;
    if (t == 0 && s.tile_counter)  // the pair kernels' work queues
        for (int k = 0; k < kPairPhases; ++k) s.tile_counter[k] = 0;
    if (t < s.n && s.contact_flag) s.contact_flag[t] = 0;
    const int c = t / s.n;
    const int i = t - c * s.n;
    const double dt = s.sc->dt;
    const double vh = s.vel.c[c][i] + (.5 * s.acc.c[c][i]) * dt;   // :84
    const double whc = s.w.c[c][i] + (.5 * s.aacc.c[c][i]) * dt;   // :87
    const double p = s.pos.c[c][i];
    const double pn = p + vh * dt;                                  // :90
    s.velh.c[c][i] = vh;
    s.wh.c[c][i] = whc;
    s.prev.c[c][i] = p;  // positions the pair distances of the previous step were taken at
    s.pos.c[c][i] = pn;
    if (s.f_pos[0]) {  // mixed form: scaled position as double-float hi + lo
        const float hi = d2f_bits(pn, s.len_shift);
        s.f_pos[c][i] = hi;
        s.f_pos[3 + c][i] = d2f_bits(pn - f2d_bits(hi) * ldexp(1.0, s.len_shift), s.len_shift);
    }
}

// ---------------------------------------------------------------- pass 2 --
// One warp per lower-triangular 32x32 block tile (X, Y), X >= Y.  Lane b
// owns sphere B = 32Y + b and walks the 32 spheres A = 32X + a of the A
// block; on the diagonal only a > b is a pair.  Tiles are independent; one
// launch covers the tiles of block columns [c0, c1) with a static stride.
// Tiles in column-major order: column Y holds tiles (Y..nb-1, Y); the first
// tile of column c has index c*nb - c(c-1)/2.
__device__ __forceinline__ long long col_offset(int nb, int c) { return (long long)c * nb - (long long)c * (c - 1) / 2; }

__device__ __forceinline__ void col_tile_coords(int nb, long long u, int& X, int& Y)
{
    const double b = 2.0 * nb + 1.0;
    int c = (int)((b - sqrt(b * b - 8.0 * (double)u)) * 0.5);
    c = max(0, min(c, nb - 1));
    while (c + 1 < nb && col_offset(nb, c + 1) <= u) ++c;
    while (c > 0 && col_offset(nb, c) > u) --c;
    Y = c;
    X = c + (int)(u - col_offset(nb, c));
}

template <bool WRITE>
__global__ void __launch_bounds__(128, 4) pair_tile_kernel(const __grid_constant__ System s, int c0, int c1,
                                                          int phase)
{
    __shared__ ABlock sA[4];
    __shared__ double sB[4][kBStageDoubles];
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    ABlock& ab = sA[wib];
    const long long nwarps = (long long)gridDim.x * 4;
    const double Ha = s.mat.Ha;
    const long long h_min_bits = __double_as_longlong(s.mat.h_min);  // h_min > 0

    // A first round of tiles in warp order; then whichever warp is free takes
    // the next tile from the launch's counter (zeroed by the drift kernel),
    // or, without a counter, the static stride.  A tile's results do not
    // depend on the warp that computes it.
    const long long u0 = col_offset(s.nb, c0), u1 = col_offset(s.nb, c1);
    int* counter = s.tile_counter ? s.tile_counter + phase : nullptr;
    for (long long u = u0 + (long long)blockIdx.x * 4 + wib; u < u1;) {
        int X, Y;
        col_tile_coords(s.nb, u, X, Y);
        const long long t = (long long)X * (X + 1) / 2 + Y;  // this tile's PE slot
        {
            const int i = X * kBlock + lane;  // < npad always
            ab.x[lane] = s.pos.c[0][i]; ab.y[lane] = s.pos.c[1][i]; ab.z[lane] = s.pos.c[2][i];
            ab.R[lane] = s.R[i]; ab.twoR[lane] = s.twoR[i]; ab.fourR[lane] = s.fourR[i];
            ab.cR3[lane] = s.cR3[i]; ab.m[lane] = s.m[i]; ab.rm[lane] = s.rm[i];
        }
        __syncwarp();
        const int B = Y * kBlock + lane;
        const bool bvalid = B < s.n;
        const double bx = s.pos.c[0][B], by = s.pos.c[1][B], bz = s.pos.c[2][B];
        const double Rb = s.R[B], twoRb = s.twoR[B], mb = s.m[B];
        const unsigned long long rmb = s.rm[B];
        const double R0 = ab.R[0];
        const bool uni = __all_sync(0xffffffffu, ab.R[lane] == R0 && Rb == R0);
        const double twoR0 = ab.twoR[0], sum0 = R0 + R0, c40 = ab.fourR[0] * R0;
        const double P0 = ab.cR3[0] * R0 * R0 * R0;
        const int a_end = min(kBlock, s.n - X * kBlock);
        double pe = 0;
        uint32_t rowbits = 0, colbits = 0;
        double* rowA = s.pairbuf + (size_t)(X * kBlock) * s.npad + B;  // + a*npad: term for A
        double* rowB = s.pairbuf + (size_t)B * s.npad + X * kBlock;    // + a: term for B

        const TileUniform tu{R0, twoR0, sum0, c40, P0};
        if (uni)
            tile_pairs<WRITE, true>(s, ab, X, Y, lane, a_end, bx, by, bz, Rb, twoRb, mb, rmb, bvalid, tu, h_min_bits,
                                    Ha, rowA, rowB, pe, rowbits, colbits, sB[wib]);
        else
            tile_pairs<WRITE, false>(s, ab, X, Y, lane, a_end, bx, by, bz, Rb, twoRb, mb, rmb, bvalid, tu, h_min_bits,
                                     Ha, rowA, rowB, pe, rowbits, colbits, sB[wib]);
        // Contact bits: row A = 32X + lane gets block Y's bits, row B gets
        // block X's bits; on the diagonal both describe row 32X + lane.
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
        if (counter) {
            int next = 0;
            if (lane == 0) next = atomicAdd(counter, 1);
            u = u0 + nwarps + __shfl_sync(0xffffffffu, next, 0);
        } else {
            u += nwarps;
        }
    }
}

// ------------------------------------------------- row sums + pass 3 ------
// Thread (c, i) continues acc_c[i] = sum over partners j ascending of
// pairbuf[c][i][j] (j != i) over the partner blocks [b0, b1), and aacc_c[i]
// likewise over the contact partners -- the order in which the reference
// adds terms to acc[i] and aacc[i].  Between segments the running sums are
// kept in acc/aacc (dead after the step's drift); the last segment does
// pass 3.  The sum is a dependent chain per (c, i), so the kernel is
// latency-bound: each thread keeps kRowBatch 16-byte loads in flight
// (register double buffering) while it adds the previous batch.
constexpr int kRowBatch = 16;
constexpr int kRowThreads = 32;

__global__ void __launch_bounds__(kRowThreads) rowsum_kernel(const __grid_constant__ System s, int b0, int b1,
                                                             int first, int last)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 3 * s.n) return;
    const int c = t / s.n;
    const int i = t - c * s.n;
    const int n = s.n;
    const size_t plane = (size_t)s.npad * s.npad;
    const double2* row = reinterpret_cast<const double2*>(s.pairbuf + c * plane + (size_t)i * s.npad);
    const int j0 = b0 * kBlock, j1 = min(b1 * kBlock, n);
    const int v0 = j0 / 2, v1 = (j1 + 1) / 2;  // double2 words covering columns [j0, j1)
    double2 cur[kRowBatch], nxt[kRowBatch];
#pragma unroll
    for (int k = 0; k < kRowBatch; ++k) cur[k] = v0 + k < v1 ? __ldcs(row + v0 + k) : make_double2(0.0, 0.0);
    double acc = first ? 0.0 : s.acc.c[c][i];
    for (int base = v0; base < v1; base += kRowBatch) {
#pragma unroll
        for (int k = 0; k < kRowBatch; ++k) {
            const int q = base + kRowBatch + k;
            nxt[k] = q < v1 ? __ldcs(row + q) : make_double2(0.0, 0.0);
        }
#pragma unroll
        for (int k = 0; k < kRowBatch; ++k) {
            const int j = 2 * (base + k);
            if (j < j1 && j != i) acc += cur[k].x;
            if (j + 1 < j1 && j + 1 != i) acc += cur[k].y;
        }
#pragma unroll
        for (int k = 0; k < kRowBatch; ++k) cur[k] = nxt[k];
    }
    double aacc = first ? 0.0 : s.aacc.c[c][i];
    const uint32_t* mrow = s.cmask + (size_t)i * s.nb;
    const double* trow = s.torqbuf + c * plane + (size_t)i * s.npad;
    for (int Y = b0; Y < b1; ++Y) {
        uint32_t wd = mrow[Y];
        while (wd) {
            const int b = __ffs(wd) - 1;
            wd &= wd - 1;
            aacc += trow[Y * kBlock + b];
        }
    }
    s.acc.c[c][i] = acc;
    s.aacc.c[c][i] = aacc;
    if (!last) return;
    const double dt = s.sc->dt;
    const double v = s.velh.c[c][i] + (.5 * acc) * dt;    // :265
    const double wv = s.wh.c[c][i] + (.5 * aacc) * dt;    // :266
    s.vel.c[c][i] = v;
    s.w.c[c][i] = wv;
    if (!isfinite(v) || !isfinite(wv) || !isfinite(s.pos.c[c][i])) atomicOr(s.status, 1u);
}

// ------------------------------------------------------ energy totals -----
constexpr int kRedThreads = 256;

// Per-sphere KE, mom, ang_mom terms (:282-285) reduced over a fixed tree:
// block b sums spheres [b*chunk, (b+1)*chunk) into red[b][0..6].
__global__ void __launch_bounds__(kRedThreads) energy_partial_kernel(const __grid_constant__ System s, int chunk)
{
    __shared__ double sh[7][kRedThreads];
    const int tid = threadIdx.x;
    double v[7] = {0, 0, 0, 0, 0, 0, 0};
    const int beg = blockIdx.x * chunk, end = min(s.n, beg + chunk);
    for (int i = beg + tid; i < end; i += kRedThreads) {
        const double m = s.m[i], moi = s.moi[i];
        const double vx = s.vel.c[0][i], vy = s.vel.c[1][i], vz = s.vel.c[2][i];
        const double wx = s.w.c[0][i], wy = s.w.c[1][i], wz = s.w.c[2][i];
        const double px = s.pos.c[0][i], py = s.pos.c[1][i], pz = s.pos.c[2][i];
        v[0] += .5 * m * (vx * vx + vy * vy + vz * vz) + .5 * moi * (wx * wx + wy * wy + wz * wz);
        v[1] += m * vx; v[2] += m * vy; v[3] += m * vz;
        const double cx = py * vz - pz * vy, cy = pz * vx - px * vz, cz = px * vy - py * vx;
        v[4] += m * cx + moi * wx; v[5] += m * cy + moi * wy; v[6] += m * cz + moi * wz;
    }
#pragma unroll
    for (int k = 0; k < 7; ++k) sh[k][tid] = v[k];
    __syncthreads();
    for (int off = kRedThreads / 2; off > 0; off >>= 1) {
        if (tid < off) {
#pragma unroll
            for (int k = 0; k < 7; ++k) sh[k][tid] += sh[k][tid + off];
        }
        __syncthreads();
    }
    if (tid < 7) s.red[blockIdx.x * 8 + tid] = sh[tid][0];
}

// Final totals: PE over all tile partials, the rest over the block partials.
__global__ void __launch_bounds__(kRedThreads) energy_final_kernel(const __grid_constant__ System s, int nred)
{
    __shared__ double sh[8][kRedThreads];
    const int tid = threadIdx.x;
    double v[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (long long t = tid; t < s.nitems; t += kRedThreads) v[0] += s.pe_tile[t];
    for (int b = tid; b < nred; b += kRedThreads)
        for (int k = 0; k < 7; ++k) v[k + 1] += s.red[b * 8 + k];
#pragma unroll
    for (int k = 0; k < 8; ++k) sh[k][tid] = v[k];
    __syncthreads();
    for (int off = kRedThreads / 2; off > 0; off >>= 1) {
        if (tid < off) {
#pragma unroll
            for (int k = 0; k < 8; ++k) sh[k][tid] += sh[k][tid + off];
        }
        __syncthreads();
    }
    if (tid < 8) s.energy[tid] = sh[tid][0];
}

// Per-sphere derived constants (exact scalings and correctly rounded
// reciprocals), computed once per upload.
__global__ void derive_kernel(const __grid_constant__ System s)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= s.npad) return;
    const double R = s.R[i], m = s.m[i], moi = s.moi[i];
    s.twoR[i] = 2 * R;
    s.fourR[i] = 4 * R;
    s.cR3[i] = s.mat.Ha / 6 * 64 * R * R * R;
    s.rm[i] = recip_of(m);
    s.inv_moi[i] = 1.0 / moi;
    if (s.f_R) {  // mixed-precision form: FP32 constants, lengths scaled by 2^-len_shift
        const float rh = d2f_bits(R, s.len_shift);
        s.f_R[i] = rh;
        s.f_Rlo[i] = d2f_bits(R - f2d_bits(rh) * ldexp(1.0, s.len_shift), s.len_shift);
        s.f_inv_m[i] = d2f_bits(1.0 / m, 0);
        s.f_inv_moi[i] = d2f_bits(1.0 / moi, 0);
    }
}

// ------------------------------------------------------ host exchange ---
struct StageArrays {
    Vec3Soa a[6];
};

// The caller's vec3[n] AoS arrays (x, y, z per sphere), one pointer each:
// host memory the kernel reads or writes directly, or device staging.
struct StagePtrs {
    const double* p[6];
};

// One thread per element of the flattened vec3[n] arrays (sphere t / 3,
// component t % 3), so that the caller-side accesses are contiguous -- they
// may cross the CPU-GPU link -- and the gather / scatter falls on the SoA
// arrays in HBM.
__global__ void stage_in_kernel(const __grid_constant__ System s, const __grid_constant__ StagePtrs src,
                                const __grid_constant__ StageArrays arr, unsigned present, unsigned check)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 3 * s.npad) return;
    const int i = t / 3, c = t - 3 * (t / 3);
    const bool real = i < s.n;
    bool finite = true;
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        const int from = (k == 5 && !(present & 32u)) ? 0 : k;  // previous positions default to the positions
        const bool have = real && ((present >> from) & 1u);
        const double v = have ? src.p[from][t] : 0.0;
        if ((check >> k) & 1u) finite = finite && isfinite(v);
        arr.a[k].c[c][i] = v;
    }
    if (!finite) atomicOr(s.status, kStatusInputNonFiniteBit);
}

__global__ void stage_out_kernel(const __grid_constant__ System s, const __grid_constant__ StagePtrs dst,
                                 const __grid_constant__ StageArrays arr, unsigned want, bool guard)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 3 * s.n) return;
    if (guard && (*s.status & kStatusInputNonFiniteBit)) return;  // the caller's arrays stay as they were
    const int i = t / 3, c = t - 3 * (t / 3);
#pragma unroll
    for (int k = 0; k < 6; ++k)
        if ((want >> k) & 1u) const_cast<double*>(dst.p[k])[t] = arr.a[k].c[c][i];
}

// ------------------------------------------------------------ launchers --
int pair_grid_blocks(long long tiles, int num_sms)
{
    long long want = (tiles + 3) / 4;
    long long cap = (long long)num_sms * 4;  // 4 CTAs (16 warps) per SM
    return (int)(want < cap ? want : cap);
}

// Block-column boundaries of the pair phases: the row-sum segment over the
// partner blocks of phase p runs on the side stream while phases p+1.. run;
// phases shrink toward the end so that little of the last segment is exposed.
int phase_bounds(int nb, int* cb)
{
    static const double frac[kPairPhases + 1] = {0.0, 1.0 / 3.0, 2.0 / 3.0, 0.85, 0.95, 1.0};
    int np = 0;
    cb[0] = 0;
    for (int p = 1; p <= kPairPhases; ++p) {
        const int c = p == kPairPhases ? nb : (int)(frac[p] * nb + 0.5);
        if (c > cb[np]) cb[++np] = c;
    }
    return np;
}

void launch_derive(const System& s, cudaStream_t st)
{
    derive_kernel<<<(s.npad + 255) / 256, 256, 0, st>>>(s);
}

void launch_stage_in(const System& s, const double* const src[6], Vec3Soa* const arr[6], unsigned present,
                     cudaStream_t st, unsigned check)
{
    StageArrays a;
    StagePtrs p;
    for (int k = 0; k < 6; ++k) {
        a.a[k] = *arr[k];
        p.p[k] = src[k];
    }
    stage_in_kernel<<<(3 * s.npad + 255) / 256, 256, 0, st>>>(s, p, a, present, check);
}

void launch_stage_out(const System& s, double* const dst[6], Vec3Soa* const arr[6], unsigned want, cudaStream_t st,
                      bool guard)
{
    StageArrays a;
    StagePtrs p;
    for (int k = 0; k < 6; ++k) {
        a.a[k] = *arr[k];
        p.p[k] = dst[k];
    }
    stage_out_kernel<<<(3 * s.n + 255) / 256, 256, 0, st>>>(s, p, a, want, guard);
}

void launch_drift(const System& s, cudaStream_t st)
{
    drift_kernel<<<(3 * s.n + kDriftThreads - 1) / kDriftThreads, kDriftThreads, 0, st>>>(s);
}

void launch_energy(const System& s, cudaStream_t st)
{
    const int nred = kRedBlocks;
    const int chunk = (s.n + nred - 1) / nred;
    energy_partial_kernel<<<nred, kRedThreads, 0, st>>>(s, chunk);
    energy_final_kernel<<<1, kRedThreads, 0, st>>>(s, nred);
}

static void launch_rowsum(const System& s, cudaStream_t st, const CUtensorMap* map, int b0, int b1, int first,
                          int last, int num_sms, bool int_adds)
{
    if (map)
        launch_rowsum_tma<double>(s, *map, b0, b1, first, last, num_sms, int_adds, st);
    else
        rowsum_kernel<<<(3 * s.n + kRowThreads - 1) / kRowThreads, kRowThreads, 0, st>>>(s, b0, b1, first, last);
}

static void launch_pair_columns(const System& s, bool write, int num_sms, cudaStream_t st, int c0, int c1, int phase)
{
    const long long tiles = ((long long)c1 * s.nb - (long long)c1 * (c1 - 1) / 2) -
                            ((long long)c0 * s.nb - (long long)c0 * (c0 - 1) / 2);
    const int pb = pair_grid_blocks(tiles, num_sms);
    if (write)
        pair_tile_kernel<true><<<pb, 128, 0, st>>>(s, c0, c1, phase);
    else
        pair_tile_kernel<false><<<pb, 128, 0, st>>>(s, c0, c1, phase);
}

void launch_step(const System& s, bool write, int num_sms, cudaStream_t st, StepTimers* tm, const StepOverlap* ov,
                 const CUtensorMap* map, bool int_adds)
{
    launch_drift(s, st);
    if (tm) cudaEventRecord(tm->ev[0], st);
    int cb[kPairPhases + 1];
    const int np = ov ? phase_bounds(s.nb, cb) : 1;
    if (np <= 1) {
        launch_pair_columns(s, write, num_sms, st, 0, s.nb, 0);
        if (tm) cudaEventRecord(tm->ev[1], st);
        launch_rowsum(s, st, map, 0, s.nb, 1, 1, num_sms, int_adds);
    } else {
        for (int p = 0; p < np; ++p) {
            launch_pair_columns(s, write, num_sms, st, cb[p], cb[p + 1], p);
            cudaEventRecord(ov->phase[p], st);
            cudaStreamWaitEvent(ov->side, ov->phase[p], 0);
            launch_rowsum(s, ov->side, map, cb[p], cb[p + 1], p == 0, p == np - 1, num_sms, int_adds);
        }
        if (tm) cudaEventRecord(tm->ev[1], st);
        cudaEventRecord(ov->join, ov->side);
        cudaStreamWaitEvent(st, ov->join, 0);
    }
    if (tm) cudaEventRecord(tm->ev[2], st);
    if (write) launch_energy(s, st);
}

}  // namespace sl
