// sl_rowsum_tma.cu -- the ordered row sums (pass 2's accumulation, then
// pass 3) with the pair terms streamed into shared memory by the bulk-copy
// (TMA) engine: rowsum_tma_kernel for the exact form's FP64 terms (tensor-
// map boxes of row-major rows).
//
// Thread (c, i) adds acc_c[i] = sum over partners j ascending of
// pairbuf[c][i][j] -- the order in which the reference adds terms to acc[i]
// and aacc[i] (ColliderSingleCore.cpp:100-103, 249-250) -- over the partner
// blocks [b0, b1), continuing the running sums kept in acc/aacc between
// segments; the last segment does pass 3 (:263-267).  FP64 terms are added
// in FP64 (the reference's own additions).
//
// Layout: one warp per (component, 32-row block), lane = row, one warp per
// CTA, so that the block scheduler spreads the warps evenly: at N=5000 the
// 471 warps land 3 or 4 to an SM (with two-warp CTAs, 84 SMs took 4 and 68
// took 2; 0.2307 -> 0.2283 ms, and 2.62 -> 2.47 ms at N=20000).  A box of
// the TMA pipeline is the warp's 32 rows x 128 bytes (16 doubles), stored
// with the 128-byte swizzle so that the lanes' 16-byte reads of their own
// rows fall in distinct bank groups (4 wavefronts per 512 bytes, the
// minimum).  kRsStages stages are in flight per warp; one lane issues the
// copies and every wait is bounded (sl_tma.cuh): a copy that does not land
// sets status bit 2 and the warp returns after draining its other copies.
// A stage is one box or two (RsStage): with one, the footprint (12 KB of
// shared memory and at most 128 registers per thread) lets 16 warps share
// an SM, so that the 3n/32 warps of a system of up to ~26,000 spheres run in
// one wave; with two, each stage wait covers twice the adds, which pays when
// the warps are few.  The stage in registers and the next one alternate
// between two register sets.
//
// Every entry of a row is added, the row's own column and the padding
// columns included: those are never written and hold +0.0 (a handle's arena
// is zeroed at creation and n is fixed per handle), and adding +0.0 leaves
// a sum that starts at +0.0 unchanged -- RN additions from +0.0 never give
// -0.0.  The chain is then additions only, which for FP64 terms the FP64
// unit bounds.
#include "sl_device.cuh"
#include "sl_kernels.h"
#include "sl_sum_exact.cuh"
#include "sl_tma.cuh"

#include <cudaTypedefs.h>
#include <mutex>

namespace sl {

namespace {

constexpr int kRsStages = 3;
constexpr int kRsWarps = 1;  // warps per CTA
constexpr int kRsBox = kBlock * 128;  // one 128-byte-wide box of 32 rows

// BPS boxes per stage: 2 when a system's warps are few (each stage wait then
// covers twice the adds), 1 when they are many (half the footprint, so that
// up to 16 warps share an SM and large systems run in one wave).
template <int BPS>
struct RsStage {
    static constexpr int kBytes = BPS * kRsBox;
    static constexpr int kWarpBytes = kRsStages * kBytes;
    static constexpr int kSmem = kRsWarps * kWarpBytes + 1024;  // + alignment slack
    static constexpr int kChunks = BPS * 8;                     // 16-byte reads per lane per stage
};

// Term type -> box width and the running-sum type a lane's 16-byte chunks
// of its row are added into.
template <typename T>
struct RsTerm;

template <>
struct RsTerm<double> {
    static constexpr int kBoxCols = 16;  // columns per box (stage)
    static constexpr CUtensorMapDataType kType = CU_TENSOR_MAP_DATA_TYPE_FLOAT64;
    // FP64 running sum: the reference's additions, in its order
    struct Acc {
        double a;
        __device__ void start(double x) { a = x; }
        __device__ void add_chunk(const uint4& u)
        {
            a += __hiloint2double((int)u.y, (int)u.x);
            a += __hiloint2double((int)u.w, (int)u.z);
        }
        __device__ void add_term(double x) { a += x; }
        __device__ double value() const { return a; }
    };
};

// Issues stage q (BPS boxes) into buffer q % NST of the warp's NST stage
// buffers, completing barrier full[q % NST].
template <typename T, int BPS, int NST = kRsStages>
__device__ __forceinline__ void rs_issue(unsigned char* buf, uint64_t* full, const CUtensorMap* map, int q, int x0,
                                         int row0)
{
    const int st = q % NST;
    unsigned char* dst = buf + st * RsStage<BPS>::kBytes;
    tma::mbar_arrive_expect_tx(&full[st], RsStage<BPS>::kBytes);
#pragma unroll
    for (int b = 0; b < BPS; ++b)
        tma::load_2d(dst + b * kRsBox, map, x0 + (q * BPS + b) * RsTerm<T>::kBoxCols, row0, &full[st]);
}

// lane's 16-byte chunk k of its own row in a stage buffer (swizzled boxes)
__device__ __forceinline__ uint4 rs_chunk(const unsigned char* stage, int lane, int k)
{
    return *reinterpret_cast<const uint4*>(stage + (k >> 3) * kRsBox + lane * 128 + (((k & 7) ^ (lane & 7)) << 4));
}

template <typename T, int BPS>
__global__ void __launch_bounds__(32 * kRsWarps, 16 / BPS) rowsum_tma_kernel(const __grid_constant__ System s,
                                                                            const __grid_constant__ CUtensorMap map,
                                                                            int b0, int b1, int first, int last)
{
    using Stage = RsStage<BPS>;
    constexpr int kStageCols = BPS * RsTerm<T>::kBoxCols;
    // stages per 32-column partner block (1 when a stage spans several blocks)
    constexpr int kSpb = kStageCols >= kBlock ? 1 : kBlock / kStageCols;
    constexpr int kBps = kStageCols >= kBlock ? kStageCols / kBlock : 1;  // partner blocks per stage
    extern __shared__ unsigned char rs_raw[];
    __shared__ __align__(8) uint64_t full_all[kRsWarps][kRsStages];
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int wg = blockIdx.x * kRsWarps + warp;  // global (component, row block) index
    if (wg >= 3 * s.nb) return;                   // no block-wide synchronisation below
    unsigned char* buf = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(rs_raw) + 1023) &
                                                          ~static_cast<uintptr_t>(1023)) +
                         warp * Stage::kWarpBytes;
    uint64_t* full = full_all[warp];
    const int c = wg / s.nb;
    const int rb = wg - c * s.nb;
    const int i = rb * kBlock + lane;  // < npad
    const int row0 = c * s.npad + rb * kBlock;
    const int x0 = b0 * kBlock;
    const int nq = (b1 - b0) * kSpb / kBps;  // callers give whole stages
    if (lane == 0) {
        for (int k = 0; k < kRsStages; ++k) tma::mbar_init(&full[k], 1);
        tma::fence_barrier_init();
        for (int q = 0; q < nq && q < kRsStages; ++q) rs_issue<T, BPS>(buf, full, &map, q, x0, row0);
    }
    __syncwarp();

    typename RsTerm<T>::Acc acc, aacc;
    acc.start(first ? 0.0 : s.acc.c[c][i]);
    aacc.start(first ? 0.0 : s.aacc.c[c][i]);
    // torque terms: contact partners only, in the same ascending order, after
    // each partner block's force terms; the contact-mask word of the next
    // partner block is loaded a block ahead
    const size_t plane = (size_t)s.npad * s.npad;
    const uint32_t* mrow = s.cmask + (size_t)i * s.nb;  // rows < npad exist; padding rows are 0
    const T* trow = reinterpret_cast<const T*>(s.torqbuf) + c * plane + (size_t)i * s.npad;
    uint32_t wnext = b1 > b0 ? mrow[b0] : 0u;
    // Software pipeline: stage q is in registers while its buffer is refilled
    // and stage q+1 is read into the other register set, so the add chain
    // never waits for a barrier or for shared memory.  The two register sets
    // alternate (the stage loop runs two stages per pass): copying the next
    // stage's registers into the current ones at the end of each stage made
    // the copies wait for the shared-memory loads, and in-order issue held
    // the next adds behind them (~18 cycles per add at N=5000).
    uint4 regs0[Stage::kChunks], regs1[Stage::kChunks];
    int waited = 0;  // first stage not yet observed complete
    bool ok = nq <= 0 || __all_sync(0xffffffffu, tma::mbar_wait(&full[0], 0));
    if (ok && nq > 0) {
#pragma unroll
        for (int k = 0; k < Stage::kChunks; ++k) regs0[k] = rs_chunk(buf, lane, k);
        waited = 1;
    }
    // stage q from cur; stage q+1 read into nxt
    auto run_stage = [&](const uint4 (&cur)[Stage::kChunks], uint4 (&nxt)[Stage::kChunks], int q) {
        // The add chain is the critical path: the bookkeeping of the stages
        // sits between its first chunks, each of which leaves the warp
        // waiting on the FP64 add latency anyway.
        acc.add_chunk(cur[0]);
        __syncwarp();  // every lane has stage q in registers: its buffer is free
        if (lane == 0 && q + kRsStages < nq) {
            tma::fence_proxy_async();
            rs_issue<T, BPS>(buf, full, &map, q + kRsStages, x0, row0);
        }
        acc.add_chunk(cur[1]);
        bool have_next = false;
        if (q + 1 < nq) {
            const int st1 = (q + 1) % kRsStages;
            ok = __all_sync(0xffffffffu, tma::mbar_wait(&full[st1], ((q + 1) / kRsStages) & 1));
            have_next = ok;
        }
        acc.add_chunk(cur[2]);
        if (have_next) {
            const int st1 = (q + 1) % kRsStages;
#pragma unroll
            for (int k = 0; k < Stage::kChunks; ++k) nxt[k] = rs_chunk(buf + st1 * Stage::kBytes, lane, k);
            waited = q + 2;
        }
#pragma unroll
        for (int pb = 0; pb < kBps; ++pb) {  // each partner block in the stage
            constexpr int kChunksPerBlock = Stage::kChunks / kBps;
#pragma unroll
            for (int k = pb * kChunksPerBlock; k < (pb + 1) * kChunksPerBlock; ++k) {
                if (k >= 3) acc.add_chunk(cur[k]);
            }
            if (q % kSpb == kSpb - 1) {  // partner block Y complete: its torque terms
                const int Y = b0 + (q / kSpb) * kBps + pb;
                uint32_t wd = wnext;
                if (Y + 1 < b1) wnext = mrow[Y + 1];
                while (wd) {
                    const int bit = __ffs(wd) - 1;
                    wd &= wd - 1;
                    aacc.add_term(trow[Y * kBlock + bit]);
                }
            }
        }
    };
    for (int q = 0; ok && q < nq; q += 2) {
        run_stage(regs0, regs1, q);
        if (!ok || q + 1 >= nq) break;
        run_stage(regs1, regs0, q + 1);
    }
    if (!ok) {
        // a wait ran out: drain the copies still in flight (each wait
        // bounded), then report.  Stages waited .. waited + kRsStages - 1 may
        // have been issued (every stage before `waited` was observed).
        const int issued = min(nq, waited + kRsStages);
        for (int qq = waited; qq < issued; ++qq) tma::mbar_wait(&full[qq % kRsStages], (qq / kRsStages) & 1);
        if (lane == 0) atomicOr(s.status, kStatusWaitTimeoutBit);
        return;
    }
    if (i >= s.n) return;
    const double fa = acc.value(), ta = aacc.value();
    s.acc.c[c][i] = fa;
    s.aacc.c[c][i] = ta;
    if (!last) return;
    const double dt = s.sc->dt;
    const double v = s.velh.c[c][i] + (.5 * fa) * dt;    // :265
    const double wv = s.wh.c[c][i] + (.5 * ta) * dt;     // :266
    s.vel.c[c][i] = v;
    s.w.c[c][i] = wv;
    if (!isfinite(v) || !isfinite(wv) || !isfinite(s.pos.c[c][i])) atomicOr(s.status, 1u);
}

// ---------------------------------------------------------------------------
// rowsum_int_kernel: the same ordered sums with each FP64 addition computed
// on the integer pipe (sl_sum_exact.cuh) instead of the FP64 unit
// (SL_ROWSUM_INT).  On GB300 it is the slower of the two at N=5000 (0.38-
// 0.40 against 0.22 ms): ~49 ALU instructions per addition at the ALU
// pipe's half rate outweigh the FP64 unit's 64-76-cycle dependent adds.
//
// Same mapping as rowsum_tma_kernel (one warp per (component, 32-row block),
// lane = row, rows streamed in 16-column TMA boxes), and a box is one chunk
// of 16 additions: the running sum at the chunk's start is kept, the 16
// additions run in the frame form, and a lane whose fast path left its
// domain (a binade prediction that failed, a binade change outside -1..+8,
// a term larger than the new sum) repeats the chunk with FP64 additions.  Both
// paths give RN(s + t) at every addition, in the reference's order, so the
// sums are the FP64 kernel's bit for bit.  Padding rows (i >= n, all terms
// +0.0, never stored) take no part in the warp's vote, so their zero sums
// cost no repeats.
constexpr int kIsStages = 4;                            // boxes in flight per warp
constexpr int kIsSmem = kRsWarps * kIsStages * kRsBox + 1024;

__device__ __forceinline__ uint64_t is_lo(const uint4& u) { return ((uint64_t)u.y << 32) | u.x; }
__device__ __forceinline__ uint64_t is_hi(const uint4& u) { return ((uint64_t)u.w << 32) | u.z; }

__global__ void __launch_bounds__(32 * kRsWarps, 8) rowsum_int_kernel(const __grid_constant__ System s,
                                                                       const __grid_constant__ CUtensorMap map,
                                                                       int b0, int b1, int first, int last)
{
    extern __shared__ unsigned char rs_raw[];
    __shared__ __align__(8) uint64_t full_all[kRsWarps][kIsStages];
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int wg = blockIdx.x * kRsWarps + warp;  // global (component, row block) index
    if (wg >= 3 * s.nb) return;                   // no block-wide synchronisation below
    unsigned char* buf = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(rs_raw) + 1023) &
                                                          ~static_cast<uintptr_t>(1023)) +
                         warp * kIsStages * kRsBox;
    uint64_t* full = full_all[warp];
    const int c = wg / s.nb;
    const int rb = wg - c * s.nb;
    const int i = rb * kBlock + lane;  // < npad
    const int row0 = c * s.npad + rb * kBlock;
    const int x0 = b0 * kBlock;
    const int nq = (b1 - b0) * (kBlock / RsTerm<double>::kBoxCols);  // 16-column boxes
    if (lane == 0) {
        for (int k = 0; k < kIsStages; ++k) tma::mbar_init(&full[k], 1);
        tma::fence_barrier_init();
        for (int q = 0; q < nq && q < kIsStages; ++q) rs_issue<double, 1, kIsStages>(buf, full, &map, q, x0, row0);
    }
    __syncwarp();
    // stage index of box q with kIsStages buffers
    auto stage_buf = [&](int q) { return buf + (q % kIsStages) * kRsBox; };

    const bool live = i < s.n;
    double slow = first ? 0.0 : s.acc.c[c][i];  // the sum whenever run holds no frame
    xs::Run run = xs::from_double(slow);
    double ta = first ? 0.0 : s.aacc.c[c][i];
    const size_t plane = (size_t)s.npad * s.npad;
    const uint32_t* mrow = s.cmask + (size_t)i * s.nb;
    const double* trow = s.torqbuf + c * plane + (size_t)i * s.npad;
    uint32_t wnext = b1 > b0 ? mrow[b0] : 0u;

    uint4 cur[8], nxt[8];
    int waited = 0;
    bool ok = nq <= 0 || __all_sync(0xffffffffu, tma::mbar_wait(&full[0], 0));
    if (ok && nq > 0) {
#pragma unroll
        for (int k = 0; k < 8; ++k) cur[k] = rs_chunk(buf, lane, k);
        waited = 1;
    }
    for (int q = 0; ok && q < nq; ++q) {
        const xs::Run r0 = run;
        float s32 = xs::shadow_of(run);
        uint32_t bad = 0;
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            xs::step(run, s32, bad, is_lo(cur[k]));
            xs::step(run, s32, bad, is_hi(cur[k]));
        }
        __syncwarp();  // every lane has box q in registers: its buffer is free
        if (lane == 0 && q + kIsStages < nq) {
            tma::fence_proxy_async();
            rs_issue<double, 1, kIsStages>(buf, full, &map, q + kIsStages, x0, row0);
        }
#pragma unroll
        for (int k = 2; k < 4; ++k) {
            xs::step(run, s32, bad, is_lo(cur[k]));
            xs::step(run, s32, bad, is_hi(cur[k]));
        }
        bool have_next = false;
        if (q + 1 < nq) {
            ok = __all_sync(0xffffffffu, tma::mbar_wait(&full[(q + 1) % kIsStages], ((q + 1) / kIsStages) & 1));
            have_next = ok;
        }
#pragma unroll
        for (int k = 4; k < 6; ++k) {
            xs::step(run, s32, bad, is_lo(cur[k]));
            xs::step(run, s32, bad, is_hi(cur[k]));
        }
        if (have_next) {
#pragma unroll
            for (int k = 0; k < 8; ++k) nxt[k] = rs_chunk(stage_buf(q + 1), lane, k);
            waited = q + 2;
        }
#pragma unroll
        for (int k = 6; k < 8; ++k) {
            xs::step(run, s32, bad, is_lo(cur[k]));
            xs::step(run, s32, bad, is_hi(cur[k]));
        }
        if (__any_sync(0xffffffffu, bad != 0 && live)) {
            if (bad != 0) {  // repeat the chunk with FP64 additions
                double v = r0.q == xs::kNoFrame ? slow : xs::to_double(r0);
#pragma unroll
                for (int k = 0; k < 8; ++k) {
                    v += __longlong_as_double((long long)is_lo(cur[k]));
                    v += __longlong_as_double((long long)is_hi(cur[k]));
                }
                slow = v;
                run = xs::from_double(v);
            }
        }
        if (q & 1) {  // partner block Y complete: its torque terms, contact partners ascending
            const int Y = b0 + (q >> 1);
            uint32_t wd = wnext;
            if (Y + 1 < b1) wnext = mrow[Y + 1];
            while (wd) {
                const int bit = __ffs(wd) - 1;
                wd &= wd - 1;
                ta += trow[Y * kBlock + bit];
            }
        }
#pragma unroll
        for (int k = 0; k < 8; ++k) cur[k] = nxt[k];
    }
    if (!ok) {
        const int issued = min(nq, waited + kIsStages);
        for (int qq = waited; qq < issued; ++qq) tma::mbar_wait(&full[qq % kIsStages], (qq / kIsStages) & 1);
        if (lane == 0) atomicOr(s.status, kStatusWaitTimeoutBit);
        return;
    }
    if (!live) return;
    const double fa = run.q == xs::kNoFrame ? slow : xs::to_double(run);
    s.acc.c[c][i] = fa;
    s.aacc.c[c][i] = ta;
    if (!last) return;
    const double dt = s.sc->dt;
    const double v = s.velh.c[c][i] + (.5 * fa) * dt;  // :265
    const double wv = s.wh.c[c][i] + (.5 * ta) * dt;   // :266
    s.vel.c[c][i] = v;
    s.w.c[c][i] = wv;
    if (!isfinite(v) || !isfinite(wv) || !isfinite(s.pos.c[c][i])) atomicOr(s.status, 1u);
}

PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder()
{
    static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* fn = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    });
    return encode;
}

// The pair-term buffer [3][npad][npad] as a 2D tensor of 3 npad rows of npad
// columns; boxes of 128 bytes x 32 rows with the 128-byte swizzle.
template <typename T>
bool make_map(const System& s, void* base, CUtensorMap* map)
{
    PFN_cuTensorMapEncodeTiled_v12000 encode = tensor_map_encoder();
    if (!encode || !base) return false;
    const cuuint64_t dims[2] = {(cuuint64_t)s.npad, (cuuint64_t)3 * s.npad};
    const cuuint64_t strides[1] = {(cuuint64_t)s.npad * sizeof(T)};
    const cuuint32_t box[2] = {(cuuint32_t)RsTerm<T>::kBoxCols, (cuuint32_t)kBlock};
    const cuuint32_t estr[2] = {1, 1};
    return encode(map, RsTerm<T>::kType, 2, base, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                  CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace

bool make_pair_map(const System& s, CUtensorMap* map)
{
    return make_map<double>(s, s.pairbuf, map) &&
           cudaFuncSetAttribute(rowsum_tma_kernel<double, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                RsStage<1>::kSmem) == cudaSuccess &&
           cudaFuncSetAttribute(rowsum_tma_kernel<double, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                RsStage<2>::kSmem) == cudaSuccess &&
           cudaFuncSetAttribute(rowsum_int_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kIsSmem) ==
               cudaSuccess;
}

template <typename T>
void launch_rowsum_tma(const System& s, const CUtensorMap& map, int b0, int b1, int first, int last, int num_sms,
                       bool int_adds, cudaStream_t st)
{
    const int ctas = (3 * s.nb + kRsWarps - 1) / kRsWarps;
    if (int_adds) {
        rowsum_int_kernel<<<ctas, 32 * kRsWarps, kIsSmem, st>>>(s, map, b0, b1, first, last);
        return;
    }
    // two-box stages while every warp fits at 8 warps per SM and the partner
    // range is whole stages; one-box stages otherwise
    const bool wide = 3 * s.nb <= 8 * num_sms && (RsTerm<T>::kBoxCols * 2 <= kBlock || (b1 - b0) % 2 == 0);
    if (wide)
        rowsum_tma_kernel<T, 2><<<ctas, 32 * kRsWarps, RsStage<2>::kSmem, st>>>(s, map, b0, b1, first, last);
    else
        rowsum_tma_kernel<T, 1><<<ctas, 32 * kRsWarps, RsStage<1>::kSmem, st>>>(s, map, b0, b1, first, last);
}

template void launch_rowsum_tma<double>(const System&, const CUtensorMap&, int, int, int, int, int, bool,
                                         cudaStream_t);

}  // namespace sl
