// sl_step_mixed64.cu -- the mixed-precision form of the step with FP64
// geometry and accumulation (SL_MODE_MIXED).
//
// What stays FP64, and where in the reference each piece sits:
//   * positions and the whole integration: drift_kernel (pass 1, shared with
//     the exact form) and pass 3 in mixed64_finish_kernel
//     (ColliderSingleCore.cpp:82-97, 263-267);
//   * the pair subtraction r = pos[B] - pos[A] (:105), one FP64 add per
//     component for every pair;
//   * for pairs closer than far_sq (1.25 radii sums or more), |r|^2, the
//     squared gap g = (R_A + R_B)^2 - |r|^2, |r| and the overlap
//     R_A + R_B - |r| = g / (R_A + R_B + |r|) (:106-110), which sets the
//     contact test, the elastic force and the clamped vdW gap; and the
//     previous-step distance test that chooses kin or kout (:119-126);
//   * per-sphere force and torque accumulation: every pair's force is
//     added into FP64 sums (two FP64 adds per component per pair, one for
//     each sphere), contact torques are summed in FP64 (:249-250, 187-188);
//   * the write-step energies: close pairs' potential in FP64, far pairs'
//     vdW bracket by the cancellation-free series (vdw_bracket, FP32) added
//     into FP64 sums, and the FP64 totals.
// FP32 does the force and torque arithmetic on the relative displacement
// r (rounded from FP64 to FP32 on the integer pipe) and the FP64 overlap:
// the vdW coefficient, elastic, gravity, sliding and rolling friction and
// the torques, in lengths scaled by 2^-len_shift.
//
// The work per pair is 9 FP64 adds (3 for r, 6 for the two spheres' sums),
// the FP32 force of a far pair (no square root: S = |r|^2 - (R_A + R_B)^2,
// T = |r|^2 - (R_A - R_B)^2), two FP32 <-> FP64 conversions per component
// done with integer instructions, and the tile sweep's shuffles.  GB300's
// FP64 pipe takes a warp instruction per ~20 cycles per SM, so the FP64
// adds bound the kernel: ~5.6 SM-cycles per pair.
//
// Accumulation order: one warp evaluates a 32 x 32 tile in a diagonal sweep
// (lane b holds column sphere B's FP64 sum; row r's FP64 sum travels one
// lane down per step to meet its next term), so each sphere's terms from a
// partner block are added in a fixed order into one FP64 partial.
// mixed64_finish_kernel adds a sphere's partials over the partner blocks in
// ascending order.  Every order is fixed, so runs repeat bit for bit.
#include "sl_device.cuh"
#include "sl_kernels.h"
#include "sl_pair_mixed.cuh"

#include <type_traits>

namespace sl {

namespace {

// Row spheres of a tile in shared memory, kRow64 doubles each: position x,
// y, z, then the scaled radius and c_vdw R^3 as two floats in one slot, then
// the FP64 radius.  A 10-word stride puts each half-warp's 8-byte loads of
// 16 different rows in 32 distinct banks.
constexpr int kRow64 = 5;
constexpr int kM64Warps = 4;
constexpr int kM64CtasPerSm = 4;  // resident CTAs per SM (the launch bounds' minimum)

__device__ __forceinline__ double pack_f2(float lo, float hi)
{
    return __hiloint2double(__float_as_int(hi), __float_as_int(lo));
}

__device__ __forceinline__ float2 unpack_f2(double d)
{
    return make_float2(__int_as_float(__double2loint(d)), __int_as_float(__double2hiint(d)));
}

// One warp per lower-triangular 32 x 32 block tile (X, Y), X >= Y: column
// lane b is sphere B = 32Y + b, row r is sphere A = 32X + r (A > B).  The
// force computed for a pair is the force on A; B receives its negative.
// Writes the FP64 partials part64[c][Y][A] (forces on sphere A from block
// Y) and part64[c][X][B], or on the diagonal one partial part64[c][X][i];
// contact bits to cmask[K][i]; contact torques (FP64) to torqbuf [A][B] and
// [B][A]; on write steps the tile's potential energy to pe_tile[t].
template <bool WRITE>
__global__ void __launch_bounds__(32 * kM64Warps, kM64CtasPerSm) mixed64_pair_kernel(const __grid_constant__ System s)
{
    __shared__ __align__(16) double rows_all[kM64Warps][kBlock * kRow64];
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    double* rows = rows_all[wib];
    const long long nwarps = (long long)gridDim.x * kM64Warps;
    const size_t plane = (size_t)s.npad * s.npad;  // torque planes
    const size_t pplane = (size_t)s.nb * s.npad;   // partial planes
    const int sh = s.len_shift;
    const float L = ldexpf(1.0f, sh);
    const float hmin_s = (float)s.mat.h_min / L;
    const float c_vdw = (float)(s.mat.Ha / 6 * 64) / L;  // dyn per unit vdw_shape
    const int nxt = (lane + 1) & (kBlock - 1);

    // A first round of tiles in warp order; then whichever warp is free
    // takes the next tile from a counter that the drift kernel zeroes.  A
    // tile's results do not depend on the warp that computes it.
    long long t = (long long)blockIdx.x * kM64Warps + wib;
    while (t < s.ntiles) {
        int X, Y;
        tile_coords(t, X, Y);
        {
            const int i = X * kBlock + lane;  // < npad
            double* row = rows + lane * kRow64;
            const float Ri = s.f_R[i];
            row[0] = s.pos.c[0][i];
            row[1] = s.pos.c[1][i];
            row[2] = s.pos.c[2][i];
            row[3] = pack_f2(Ri, c_vdw * (Ri * Ri * Ri));
            row[4] = s.R[i];
        }
        __syncwarp();
        const int B = Y * kBlock + lane;
        const bool bvalid = B < s.n;
        const double bx = s.pos.c[0][B], by = s.pos.c[1][B], bz = s.pos.c[2][B];
        const float Rbs = s.f_R[B];
        const float Rb3 = Rbs * Rbs * Rbs;
        const int nA = s.n - X * kBlock;  // rows r < nA are spheres
        double pe = 0.0;       // close pairs' potential (FP64)
        double pe_far = 0.0;   // far pairs' vdW brackets, times -Ha/6 at the end
        uint32_t colbits = 0;
        double ax = 0.0, ay = 0.0, az = 0.0;     // running sum of row (lane + k) mod 32 at step k
        double bsx = 0.0, bsy = 0.0, bsz = 0.0;  // sphere B's sum
        // FULL: a tile off the diagonal whose rows and columns are all spheres
        auto sweep = [&](auto full_tag) {
            constexpr bool FULL = decltype(full_tag)::value;
#pragma unroll 2
            for (int k = 0; k < kBlock; ++k) {
                const int r = (lane + k) & (kBlock - 1);
                const bool valid = FULL || (bvalid && r < nA && (X != Y || lane < r));
                const double* q = rows + r * kRow64;
                // FP64 pair subtraction (:105)
                const double rx64 = bx - q[0];
                const double ry64 = by - q[1];
                const double rz64 = bz - q[2];
                const float2 ra = unpack_f2(q[3]);
                const float Ras = ra.x;
                // the FP32 force arithmetic works on r rounded to FP32 (scaled)
                const float rx = d2f_bits(rx64, sh);
                const float ry = d2f_bits(ry64, sh);
                const float rz = d2f_bits(rz64, sh);
                const float d2 = fmaf(rx, rx, fmaf(ry, ry, rz * rz));
                const float sumR = Ras + Rbs, difR = Ras - Rbs;
                const float sum2 = sumR * sumR;
                // far pair out of contact, h above the clamp h_min: the vdW
                // force (:205-226) Ra^3 Rb^3 (h + Ra + Rb) / (S^2 T^2) along
                // r / |r| with h + Ra + Rb = |r|, S = |r|^2 - (Ra + Rb)^2 and
                // T = |r|^2 - (Ra - Rb)^2, without a square root
                const float S = d2 - sum2;
                const float T = fmaf(-difR, difR, d2);
                const float P = S * T;
                const float fr = (ra.y * Rb3) * rcp_approx(P * P);  // |F| / |r|
                float fx = fr * rx, fy = fr * ry, fz = fr * rz;
                const bool closep = d2 < s.far_sq * sum2;
                if (valid && closep) {
                    const int A = X * kBlock + r;
                    // FP64 |r|^2, squared gap, |r| and overlap (:106-110)
                    const double d2_64 = fma(rx64, rx64, fma(ry64, ry64, rz64 * rz64));
                    const double Ra64 = q[4], Rb64 = s.R[B];
                    const double sum64 = Ra64 + Rb64;
                    const double gap2 = fma(sum64, sum64, -d2_64);
                    const double dist64 = sqrt(d2_64);
                    const double ovl64 = gap2 / (sum64 + dist64);
                    const float dist_s = d2f_bits(dist64, sh);
                    const float ovl_s = d2f_bits(ovl64, sh);
                    const float inv_d = 1.0f / dist_s;
                    const float nx = rx * inv_d, ny = ry * inv_d, nz = rz * inv_d;
                    if (gap2 > 0.0) {  // contact (:119)
                        colbits |= 1u << r;
                        const ContactIn in = gather_contact(s, A, B);
                        const ContactF o = contact_mixed(in, s.mat, sh, d2_64, nx, ny, nz, dist_s * L, ovl_s * L,
                                                         Ras, Rbs);
                        fx = o.fx; fy = o.fy; fz = o.fz;
                        double* ta = s.torqbuf + (size_t)A * s.npad + B;
                        double* tb = s.torqbuf + (size_t)B * s.npad + A;
                        ta[0] = f2d_bits(o.tax); ta[plane] = f2d_bits(o.tay); ta[2 * plane] = f2d_bits(o.taz);
                        tb[0] = f2d_bits(o.tbx); tb[plane] = f2d_bits(o.tby); tb[2 * plane] = f2d_bits(o.tbz);
                        if (WRITE) pe += pair_pe_fp64(s.mat, Ra64, Rb64, gap2, d2_64, true, o.k);
                    } else {
                        const float hn = fmaxf(-ovl_s, hmin_s);  // :211-215
                        const float f = c_vdw * vdw_shape(hn, Ras, Rbs);
                        fx = f * nx; fy = f * ny; fz = f * nz;
                        if (WRITE) pe += pair_pe_fp64(s.mat, Ra64, Rb64, gap2, d2_64, false, 0.0);
                    }
                } else if (WRITE && valid) {
                    pe_far += f2d_bits(vdw_bracket(d2, Ras, Rbs));
                }
                if (!FULL && !valid) fx = fy = fz = 0.0f;
                // FP64 accumulation of both spheres' sums (:249-250)
                const double fxd = f2d_bits(fx), fyd = f2d_bits(fy), fzd = f2d_bits(fz);
                ax += fxd; ay += fyd; az += fzd;
                bsx += fxd; bsy += fyd; bsz += fzd;
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
        double* Pt = s.part64;
        if (X == Y) {  // sphere iA == B: partners j < i as A (row), j > i as B (column)
            const size_t o = (size_t)X * s.npad + iA;
            Pt[o] = ax - bsx;
            Pt[o + pplane] = ay - bsy;
            Pt[o + 2 * pplane] = az - bsz;
            s.cmask[o] = rowbits | colbits;
            if (rowbits | colbits) s.contact_flag[iA] = 1;
        } else {
            const size_t oa = (size_t)Y * s.npad + iA, ob = (size_t)X * s.npad + B;
            Pt[oa] = ax; Pt[oa + pplane] = ay; Pt[oa + 2 * pplane] = az;
            Pt[ob] = -bsx; Pt[ob + pplane] = -bsy; Pt[ob + 2 * pplane] = -bsz;
            s.cmask[oa] = rowbits;
            s.cmask[ob] = colbits;
            if (rowbits) s.contact_flag[iA] = 1;  // every writer stores 1
            if (colbits) s.contact_flag[B] = 1;
        }
        if (WRITE) {
            pe += -s.mat.Ha / 6 * pe_far;
            for (int off = 16; off > 0; off >>= 1) pe += __shfl_xor_sync(0xffffffffu, pe, off);
            if (lane == 0) s.pe_tile[t] = pe;
        }
        __syncwarp();
        int next = 0;
        if (lane == 0) next = atomicAdd(s.tile_counter, 1);
        t = nwarps + __shfl_sync(0xffffffffu, next, 0);
    }
}

constexpr int kFin64Slices = 8;

// Per-sphere totals, then pass 3.  Block = 32 spheres (lanes) x
// kFin64Slices warps; warp w adds partner blocks [nb w / S, nb (w+1) / S)
// of its lane's sphere in ascending order: the FP64 force partials
// part64[c][K][i] (coalesced along i) and the FP64 torques of contact
// partners (bits of cmask[K][i], ascending).  Warp c < 3 then adds
// component c's slices in order and integrates it in FP64: acc = F / m,
// aacc = torque / moi (the reference divides each pair's term, :249-250,
// 187-188; here the sums are divided once), then
// ColliderSingleCore.cpp:263-267.
__global__ void __launch_bounds__(32 * kFin64Slices) mixed64_finish_kernel(const __grid_constant__ System s)
{
    __shared__ double fs[kFin64Slices][6][kBlock];  // (slice, force x y z, torque x y z, sphere)
    const int lane = threadIdx.x & 31;
    const int w = threadIdx.x >> 5;
    const int i = blockIdx.x * kBlock + lane;  // < npad
    const int K0 = (int)((long long)s.nb * w / kFin64Slices);
    const int K1 = (int)((long long)s.nb * (w + 1) / kFin64Slices);
    const size_t pplane = (size_t)s.nb * s.npad;
    const size_t plane = (size_t)s.npad * s.npad;
    const double* p = s.part64 + i;
    const uint32_t* mk = s.cmask + i;
    const bool any_contact = i < s.n && s.contact_flag[i] != 0;
    const double* tb = s.torqbuf + (size_t)i * s.npad;
    double f[3] = {0.0, 0.0, 0.0};
    double tq[3] = {0.0, 0.0, 0.0};
    auto torques = [&](uint32_t wd, int K) {
        while (wd) {
            const int j = K * kBlock + __ffs(wd) - 1;
            wd &= wd - 1;
#pragma unroll
            for (int c = 0; c < 3; ++c) tq[c] += tb[j + c * plane];
        }
    };
    constexpr int U = 8;  // loads in flight per array
    int K = K0;
    for (; K + U <= K1; K += U) {
        double v[3][U];
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
            for (int c = 0; c < 3; ++c) f[c] += v[c][u];
            torques(m[u], K + u);
        }
    }
    for (; K < K1; ++K) {
        const size_t o = (size_t)K * s.npad;
#pragma unroll
        for (int c = 0; c < 3; ++c) f[c] += __ldcs(p + o + c * pplane);
        torques(any_contact ? __ldcs(mk + o) : 0u, K);
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        fs[w][c][lane] = f[c];
        fs[w][3 + c][lane] = tq[c];
    }
    __syncthreads();
    if (w >= 3 || i >= s.n) return;
    const int c = w;
    double F = 0.0, Q = 0.0;
#pragma unroll
    for (int ww = 0; ww < kFin64Slices; ++ww) {
        F += fs[ww][c][lane];
        Q += fs[ww][3 + c][lane];
    }
    const double acc = F / s.m[i];
    const double aacc = Q / s.moi[i];
    const double dt = s.sc->dt;
    const double v = s.velh.c[c][i] + (.5 * acc) * dt;   // :265
    const double wv = s.wh.c[c][i] + (.5 * aacc) * dt;  // :266
    s.acc.c[c][i] = acc;
    s.aacc.c[c][i] = aacc;
    s.vel.c[c][i] = v;
    s.w.c[c][i] = wv;
    if (!isfinite(v) || !isfinite(wv) || !isfinite(s.pos.c[c][i])) atomicOr(s.status, 1u);
}

}  // namespace

void launch_step_mixed64(const System& s, bool write, int num_sms, cudaStream_t st, StepTimers* tm)
{
    launch_drift(s, st);
    if (tm) cudaEventRecord(tm->ev[0], st);
    const long long want = (s.ntiles + kM64Warps - 1) / kM64Warps;
    const long long cap = (long long)num_sms * kM64CtasPerSm;  // one wave of persistent warps
    const int pb = (int)(want < cap ? want : cap);
    if (write)
        mixed64_pair_kernel<true><<<pb, 32 * kM64Warps, 0, st>>>(s);
    else
        mixed64_pair_kernel<false><<<pb, 32 * kM64Warps, 0, st>>>(s);
    if (tm) cudaEventRecord(tm->ev[1], st);
    mixed64_finish_kernel<<<s.nb, 32 * kFin64Slices, 0, st>>>(s);
    if (tm) cudaEventRecord(tm->ev[2], st);
    if (write) launch_energy(s, st);
}

}  // namespace sl
