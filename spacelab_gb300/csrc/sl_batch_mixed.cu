// sl_batch_mixed.cu -- batched solver in the mixed-precision form: the same
// persistent work-queue launch as sl_batch.cu, with the pair math of the
// mixed form: far pairs entirely in FP32 (no square root), close pairs with
// double-float (sl_df.cuh) displacement, |r|^2 and squared gap from the
// double-float positions the drift writes; FP32 forces and torques; FP64
// kin/kout test and write-step potential energy of close pairs from the
// FP64 positions (far pairs: the FP32 series of vdw_bracket).  The
// non-contact pair path issues no FP64 instruction.  Two pair passes over
// each instance's Z-ordered slots (sl_batch.h): the pair-tile pass (shape
// tile 0, every pair once, per-CTA partial sums) and the per-sphere loop
// (j-tiles of 32/64/128, every pair from both sides, FP32 sums per j-tile
// joined in compensated per-sphere totals).
#include "sl_batch.h"
#include "sl_batch_common.cuh"
#include "sl_df.cuh"
#include "sl_pair_mixed.cuh"

#include <type_traits>

namespace sl {

namespace {

using batch::drift;
using batch::kick;

template <int TILE>
struct JTileM {
    float4 q0[TILE];  // scaled position hi x, y, z and scaled radius R
    float4 q1[TILE];  // scaled position lo x, y, z and R^3
    float Rlo[TILE];  // the radius's double-float lo part
    int idx[TILE];    // the sphere's index in the instance (its slot's perm entry)
};

// |pos[gB] - pos[gA]|^2 in FP64, the previous-step formula of contact_mixed
__device__ __forceinline__ double fp64_d2(const Batch& b, int gA, int gB)
{
    const double rx = b.pos.c[0][gB] - b.pos.c[0][gA];
    const double ry = b.pos.c[1][gB] - b.pos.c[1][gA];
    const double rz = b.pos.c[2][gB] - b.pos.c[2][gA];
    return fma(rx, rx, fma(ry, ry, rz * rz));
}

// Thread i walks partners j through shared-memory j-tiles and adds the
// force on i, F_ij, into a plain FP32 sum per tile, which joins i's
// compensated total; acc[i] = total / m[i].  A far pair
// (|r| >= 1.25 (R_i + R_j) or more, far_sq) takes the FP32 path of the all-pairs mixed
// kernel: vdW along
// r = pos[j] - pos[i] without a square root, (c R_i^3 R_j^3) r / (S T)^2 with
// S = |r|^2 - (R_i + R_j)^2 and T = |r|^2 - (R_i - R_j)^2; a near pair the
// double-float geometry and, in contact, contact_mixed in the pair's own
// (A, B) orientation (ColliderSingleCore.cpp:104-253).
template <int TILE, bool WRITE>
__device__ double pair_pass_mixed(const Batch& b, int off, int n, const Material& M, double kin, double kout,
                                  JTileM<TILE>& jt)
{
    const int sh = b.len_shift;
    const float L = ldexpf(1.0f, sh);
    const float hmin_s = (float)M.h_min / L;
    const float c_vdw = (float)(M.Ha / 6 * 64) / L;
    double pe = 0;
    df::Sum pe_far{0.0f, 0.0f};  // far pairs' vdW brackets (write steps, i = A)
    for (int ibase = 0; ibase < n; ibase += blockDim.x) {
        const bool active = ibase + threadIdx.x < n;
        const int si = off + (active ? ibase + threadIdx.x : 0);  // slot: Z-order, a warp's spheres are close
        const int gi = b.perm[si];
        const int i = gi - off;
        const float pih[3] = {b.f_pos[0][si], b.f_pos[1][si], b.f_pos[2][si]};
        const float pil[3] = {b.f_pos[3][si], b.f_pos[4][si], b.f_pos[5][si]};
        const float Ri = b.f_R[si], Rilo = b.f_Rlo[si];
        const float cR3i = c_vdw * (Ri * Ri * Ri);
        const float imoii = b.f_inv_moi[si];
        df::Sum ax{0.0f, 0.0f}, ay{0.0f, 0.0f}, az{0.0f, 0.0f};
        double tx = 0, ty = 0, tz = 0;
        for (int jbase = 0; jbase < n; jbase += TILE) {
            for (int t = threadIdx.x; t < TILE; t += blockDim.x) {
                const int j = jbase + t;
                if (j < n) {
                    const int g = off + j;  // slot
                    const float r = b.f_R[g];
                    jt.q0[t] = make_float4(b.f_pos[0][g], b.f_pos[1][g], b.f_pos[2][g], r);
                    jt.q1[t] = make_float4(b.f_pos[3][g], b.f_pos[4][g], b.f_pos[5][g], r * r * r);
                    jt.Rlo[t] = b.f_Rlo[g];
                    jt.idx[t] = b.perm[g] - off;
                }
            }
            __syncthreads();
            if (active) {
                // close pair in slot jbase + t: double-float geometry, contact or
                // clamped vdW in the pair's (A, B) orientation; the force on i
                auto close_pair = [&](int t, float& fx, float& fy, float& fz) {
                    const int j = jt.idx[t];
                    const bool iA = i > j;
                    const float4 q0 = jt.q0[t], q1 = jt.q1[t];
                    const float Rj = q0.w;
                    // r = pos[B] - pos[A] in double-float; the sign flips with the orientation
                    const df::F2 pj[3] = {{q0.x, q1.x}, {q0.y, q1.y}, {q0.z, q1.z}};
                    df::F2 r3[3];
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        const df::F2 pi{pih[c], pil[c]};
                        r3[c] = iA ? df::sub(pj[c], pi) : df::sub(pi, pj[c]);
                    }
                    const df::F2 dd2 = df::add(df::add(df::sqr(r3[0]), df::sqr(r3[1])), df::sqr(r3[2]));
                    const df::F2 sum = df::add({Ri, Rilo}, {Rj, jt.Rlo[t]});
                    const df::F2 gap2 = df::sub(df::sqr(sum), dd2);
                    const float Ras = iA ? Ri : Rj, Rbs = iA ? Rj : Ri;
                    const float d2s = dd2.hi;
                    const float inv_d = rsqrtf(d2s);
                    const float dist_s = d2s * inv_d;
                    const float ovl_s = __fdividef(gap2.hi, Ras + Rbs + dist_s);
                    const float nx = r3[0].hi * inv_d, ny = r3[1].hi * inv_d, nz = r3[2].hi * inv_d;
                    float Fx, Fy, Fz;  // force on A
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
                        const ContactF o = contact_mixed(in, M, sh, d2_64, nx, ny, nz, dist_s * L, ovl_s * L, Ras, Rbs);
                        Fx = o.fx; Fy = o.fy; Fz = o.fz;
                        const float qx = iA ? o.tax : o.tbx, qy = iA ? o.tay : o.tby, qz = iA ? o.taz : o.tbz;
                        tx += f2d_bits(qx * imoii); ty += f2d_bits(qy * imoii); tz += f2d_bits(qz * imoii);
                        if (WRITE && iA) {
                            const double sum64 = b.R[gA] + b.R[gB];
                            pe += pair_pe_fp64(M, b.R[gA], b.R[gB], fma(sum64, sum64, -d2_64), d2_64, true, o.k);
                        }
                    } else {
                        const float h = fmaxf(-ovl_s, hmin_s);
                        const float f = c_vdw * vdw_shape(h, Ras, Rbs);
                        Fx = f * nx; Fy = f * ny; Fz = f * nz;
                        if (WRITE && iA) {
                            const double d2_64 = fp64_d2(b, gA, gB), sum64 = b.R[gA] + b.R[gB];
                            pe += pair_pe_fp64(M, b.R[gA], b.R[gB], fma(sum64, sum64, -d2_64), d2_64, false, 0.0);
                        }
                    }
                    // acc[A] += F/m[A]; acc[B] -= F/m[B]
                    fx = iA ? Fx : -Fx; fy = iA ? Fy : -Fy; fz = iA ? Fz : -Fz;
                };
                // far pair (or not a pair): its force on i, 0 where it is not
                // far; returns whether it is close
                auto far_pair = [&](int t, float& fx, float& fy, float& fz) {
                    const int j = jt.idx[t];
                    const bool valid = j != i;
                    const float4 q0 = jt.q0[t], q1 = jt.q1[t];
                    const float Rj = q0.w;
                    const float rx = (q0.x - pih[0]) + (q1.x - pil[0]);
                    const float ry = (q0.y - pih[1]) + (q1.y - pil[1]);
                    const float rz = (q0.z - pih[2]) + (q1.z - pil[2]);
                    const float d2 = fmaf(rx, rx, fmaf(ry, ry, rz * rz));
                    const float sumR = Ri + Rj, difR = Ri - Rj;
                    const float sum2 = sumR * sumR;
                    const float S = d2 - sum2;
                    const float T = fmaf(-difR, difR, d2);
                    const float P = S * T;
                    const float fr = (cR3i * q1.w) * rcp_approx(P * P);
                    const bool close = d2 < b.far_sq * sum2;
                    const bool use = valid && !close;
                    fx = use ? fr * rx : 0.0f;
                    fy = use ? fr * ry : 0.0f;
                    fz = use ? fr * rz : 0.0f;
                    if (WRITE && use && i > j) pe_far.add(vdw_bracket(d2, Ri, Rj));
                    return valid && close;
                };
                const int jend = min(TILE, n - jbase);
                float sx = 0, sy = 0, sz = 0;  // this tile's forces on i
                int t = 0;
                // four partners at a time, so that their far-pair arithmetic
                // interleaves; the close ones after, in one branch
                for (; t + 4 <= jend; t += 4) {
                    uint32_t closem = 0;
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        float fx, fy, fz;
                        closem |= (uint32_t)far_pair(t + u, fx, fy, fz) << u;
                        sx += fx; sy += fy; sz += fz;
                    }
                    if (closem) {
#pragma unroll 1
                        for (int u = 0; u < 4; ++u)
                            if ((closem >> u) & 1u) {
                                float fx, fy, fz;
                                close_pair(t + u, fx, fy, fz);
                                sx += fx; sy += fy; sz += fz;
                            }
                    }
                }
                for (; t < jend; ++t) {
                    float fx, fy, fz;
                    if (far_pair(t, fx, fy, fz)) close_pair(t, fx, fy, fz);
                    sx += fx; sy += fy; sz += fz;
                }
                ax.add(sx); ay.add(sy); az.add(sz);
            }
            __syncthreads();
        }
        if (active) {
            const double imi = f2d_bits(b.f_inv_m[si]);
            b.acc.c[0][gi] = (f2d_bits(ax.s) + f2d_bits(ax.c)) * imi;
            b.acc.c[1][gi] = (f2d_bits(ay.s) + f2d_bits(ay.c)) * imi;
            b.acc.c[2][gi] = (f2d_bits(az.s) + f2d_bits(az.c)) * imi;
            b.aacc.c[0][gi] = tx; b.aacc.c[1][gi] = ty; b.aacc.c[2][gi] = tz;
        }
    }
    if (WRITE) pe += -M.Ha / 6 * (f2d_bits(pe_far.s) + f2d_bits(pe_far.c));
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

// ---------------------------------------------------------------------------
// Pair-tile pass: every unordered pair once.  The CTA's warps take the
// instance's lower-triangular 32 x 32 slot-block tiles in turn and sweep
// each diagonally as the all-pairs mixed kernel does (sl_step_mixed.cu): at
// step k lane b takes (row (b + k) mod 32, column b), its column sum stays in
// a register and each row sum moves one lane down per step.  A tile writes one
// FP32 partial per sphere and component -- forces and torques -- to the CTA's
// scratch part[6][nb][np] (slot-indexed), and the CTA then adds each sphere's
// partials over the partner blocks in ascending order in compensated sums.
// Torques exist only in contact: a row sphere's arrive by shared-memory adds
// (one lane per row in a step, the steps in program order, so the order is
// fixed), a column sphere's in a register.
constexpr int kRowStrideT = 12;  // floats per row sphere: hi xyz R | lo xyz cR3 | Rlo 1/m 1/moi index
constexpr int kTileWarps = 16;  // up to 512 threads: a large instance can have a whole SM

struct TileSmem {
    float rows[kTileWarps][kBlock * kRowStrideT];
    float rowtq[kTileWarps][3 * kBlock];
};

template <bool WRITE>
__device__ double tile_pass_mixed(const Batch& b, int off, int n, const Material& M, double kin, double kout,
                                  TileSmem& sm)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    const int sh = b.len_shift;
    const float L = ldexpf(1.0f, sh);
    const float hmin_s = (float)M.h_min / L;
    const float c_vdw = (float)(M.Ha / 6 * 64) / L;
    const int nbk = (n + kBlock - 1) / kBlock;
    const long long ntiles = (long long)nbk * (nbk + 1) / 2;
    float* part = b.part + (size_t)blockIdx.x * b.part_cta;
    const size_t pplane = (size_t)b.part_nb * b.part_np;
    float* rows = sm.rows[warp];
    float* rowtq = sm.rowtq[warp];
    const int nxt = (lane + 1) & (kBlock - 1);
    double pe = 0;
    df::Sum pe_far{0.0f, 0.0f};  // far pairs' vdW brackets (write steps)
    for (long long t = warp; t < ntiles; t += nwarps) {
        int X, Y;
        tile_coords(t, X, Y);
        {
            const int sA = off + min(X * kBlock + lane, n - 1);  // slot (padding rows repeat the last)
            const float Ri = b.f_R[sA];
            float* row = rows + lane * kRowStrideT;
            *reinterpret_cast<float4*>(row) = make_float4(b.f_pos[0][sA], b.f_pos[1][sA], b.f_pos[2][sA], Ri);
            *reinterpret_cast<float4*>(row + 4) =
                make_float4(b.f_pos[3][sA], b.f_pos[4][sA], b.f_pos[5][sA], c_vdw * (Ri * Ri * Ri));
            row[8] = b.f_Rlo[sA];
            row[9] = b.f_inv_m[sA];
            row[10] = b.f_inv_moi[sA];
            row[11] = __int_as_float(b.perm[sA] - off);
            rowtq[lane] = 0.0f; rowtq[kBlock + lane] = 0.0f; rowtq[2 * kBlock + lane] = 0.0f;
        }
        __syncwarp();
        const int sB = Y * kBlock + lane;  // slot in the instance
        const bool bvalid = sB < n;
        const int gBs = off + min(sB, n - 1);
        const float bx = b.f_pos[0][gBs], by = b.f_pos[1][gBs], bz = b.f_pos[2][gBs];
        const float bxl = b.f_pos[3][gBs], byl = b.f_pos[4][gBs], bzl = b.f_pos[5][gBs];
        const float Rbs = b.f_R[gBs], Rblo = b.f_Rlo[gBs], inv_mb = b.f_inv_m[gBs], imoib = b.f_inv_moi[gBs];
        const int iB = b.perm[gBs] - off;  // the column sphere's index in the instance
        const float Rb3 = Rbs * Rbs * Rbs;
        const int nA = n - X * kBlock;
        float ax = 0, ay = 0, az = 0;        // running sum of row (lane + k) mod 32 at step k
        float bsx = 0, bsy = 0, bsz = 0;     // the column sphere's force sum
        float ctx = 0, cty = 0, ctz = 0;     // the column sphere's torque sum
        // close pair (row r, this lane's column): double-float geometry, then
        // the contact branch in the reference's orientation (A = the larger
        // index in the instance) or the clamped vdW; the force on the row sphere
        auto close_pair = [&](int r, float& fx, float& fy, float& fz) {
            const float4 q0 = *reinterpret_cast<const float4*>(rows + r * kRowStrideT);
            const float4 q1 = *reinterpret_cast<const float4*>(rows + r * kRowStrideT + 4);
            const float Ras = q0.w;
            const int iA = __float_as_int(rows[r * kRowStrideT + 11]);
            const df::F2 drx = df::sub({bx, bxl}, {q0.x, q1.x});
            const df::F2 dry = df::sub({by, byl}, {q0.y, q1.y});
            const df::F2 drz = df::sub({bz, bzl}, {q0.z, q1.z});
            const df::F2 dd2 = df::add(df::add(df::sqr(drx), df::sqr(dry)), df::sqr(drz));
            const df::F2 sum = df::add({Ras, rows[r * kRowStrideT + 8]}, {Rbs, Rblo});
            const df::F2 gap2 = df::sub(df::sqr(sum), dd2);
            const float d2s = dd2.hi;
            const float inv_dn = rsqrtf(d2s);
            const float dist_s = d2s * inv_dn;
            const float ovl_s = __fdividef(gap2.hi, Ras + Rbs + dist_s);
            const float nx = drx.hi * inv_dn, ny = dry.hi * inv_dn, nz = drz.hi * inv_dn;  // row -> column
            const bool rowA = iA > iB;
            const int gA = off + (rowA ? iA : iB), gB = off + (rowA ? iB : iA);
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
                const float sg = rowA ? 1.0f : -1.0f;  // unit vector A -> B
                const ContactF o = contact_mixed(in, M, sh, d2_64, sg * nx, sg * ny, sg * nz, dist_s * L, ovl_s * L,
                                                 rowA ? Ras : Rbs, rowA ? Rbs : Ras);
                fx = sg * o.fx; fy = sg * o.fy; fz = sg * o.fz;  // o.f acts on A; B takes -o.f
                const float imoia = rows[r * kRowStrideT + 10];
                atomicAdd(&rowtq[r], (rowA ? o.tax : o.tbx) * imoia);
                atomicAdd(&rowtq[kBlock + r], (rowA ? o.tay : o.tby) * imoia);
                atomicAdd(&rowtq[2 * kBlock + r], (rowA ? o.taz : o.tbz) * imoia);
                ctx += (rowA ? o.tbx : o.tax) * imoib;
                cty += (rowA ? o.tby : o.tay) * imoib;
                ctz += (rowA ? o.tbz : o.taz) * imoib;
                if (WRITE) {
                    const double sum64 = b.R[gA] + b.R[gB];
                    pe += pair_pe_fp64(M, b.R[gA], b.R[gB], fma(sum64, sum64, -d2_64), d2_64, true, o.k);
                }
                return;
            }
            const float hn = fmaxf(-ovl_s, hmin_s);
            const float f = c_vdw * vdw_shape(hn, Ras, Rbs);
            fx = f * nx; fy = f * ny; fz = f * nz;
            if (WRITE) {
                const double d2_64 = fp64_d2(b, gA, gB), sum64 = b.R[gA] + b.R[gB];
                pe += pair_pe_fp64(M, b.R[gA], b.R[gB], fma(sum64, sum64, -d2_64), d2_64, false, 0.0);
            }
        };
        auto sweep = [&](auto full_tag) {
            constexpr bool FULL = decltype(full_tag)::value;
#pragma unroll 2
            for (int k = 0; k < kBlock; ++k) {
                const int r = (lane + k) & (kBlock - 1);
                const bool valid = FULL || (bvalid && r < nA && (X != Y || lane < r));
                const float4 q0 = *reinterpret_cast<const float4*>(rows + r * kRowStrideT);
                const float4 q1 = *reinterpret_cast<const float4*>(rows + r * kRowStrideT + 4);
                const float Ras = q0.w;
                // far pair: vdW without a square root (sl_step_mixed.cu)
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
                const bool close = d2 < b.far_sq * sum2;
                if (valid && close) close_pair(r, fx, fy, fz);
                if (WRITE && valid && !close) pe_far.add(vdw_bracket(d2, Ras, Rbs));
                if (!FULL && !valid) fx = fy = fz = 0.0f;
                ax += fx; ay += fy; az += fz;
                bsx += fx; bsy += fy; bsz += fz;
                ax = __shfl_sync(0xffffffffu, ax, nxt);
                ay = __shfl_sync(0xffffffffu, ay, nxt);
                az = __shfl_sync(0xffffffffu, az, nxt);
            }
        };
        if (X != Y && (X + 1) * kBlock <= n)
            sweep(std::true_type{});
        else
            sweep(std::false_type{});
        __syncwarp();  // the row torques' shared-memory adds
        // lane l holds row l's force sum (rows and columns beyond n hold 0)
        const int sAl = X * kBlock + lane;
        const float ima = rows[lane * kRowStrideT + 9];
        const float rtx = rowtq[lane], rty = rowtq[kBlock + lane], rtz = rowtq[2 * kBlock + lane];
        if (X == Y) {  // the same sphere: partners before it in slot order (row), after it (column)
            const size_t o = (size_t)X * b.part_np + sAl;
            part[o] = fmaf(ima, ax, -inv_mb * bsx);
            part[o + pplane] = fmaf(ima, ay, -inv_mb * bsy);
            part[o + 2 * pplane] = fmaf(ima, az, -inv_mb * bsz);
            part[o + 3 * pplane] = rtx + ctx;
            part[o + 4 * pplane] = rty + cty;
            part[o + 5 * pplane] = rtz + ctz;
        } else {
            const size_t oa = (size_t)Y * b.part_np + sAl, ob = (size_t)X * b.part_np + sB;
            part[oa] = ima * ax; part[oa + pplane] = ima * ay; part[oa + 2 * pplane] = ima * az;
            part[oa + 3 * pplane] = rtx; part[oa + 4 * pplane] = rty; part[oa + 5 * pplane] = rtz;
            part[ob] = -inv_mb * bsx; part[ob + pplane] = -inv_mb * bsy; part[ob + 2 * pplane] = -inv_mb * bsz;
            part[ob + 3 * pplane] = ctx; part[ob + 4 * pplane] = cty; part[ob + 5 * pplane] = ctz;
        }
        __syncwarp();
    }
    if (WRITE) pe += -M.Ha / 6 * (f2d_bits(pe_far.s) + f2d_bits(pe_far.c));
    return pe;
}

// The CTA's per-sphere totals from the tile partials (partner blocks in
// ascending order, compensated sums), to acc and aacc in the caller's order.
__device__ __forceinline__ void tile_totals(const Batch& b, int off, int n)
{
    const int nbk = (n + kBlock - 1) / kBlock;
    const float* part = b.part + (size_t)blockIdx.x * b.part_cta;
    const size_t pplane = (size_t)b.part_nb * b.part_np;
    for (int p = threadIdx.x; p < n; p += blockDim.x) {
        df::Sum tot[6] = {{0.0f, 0.0f}, {0.0f, 0.0f}, {0.0f, 0.0f}, {0.0f, 0.0f}, {0.0f, 0.0f}, {0.0f, 0.0f}};
        for (int K = 0; K < nbk; ++K) {
            const float* e = part + (size_t)K * b.part_np + p;
#pragma unroll
            for (int q = 0; q < 6; ++q) tot[q].add(e[q * pplane]);
        }
        const int g = b.perm[off + p];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            b.acc.c[c][g] = f2d_bits(tot[c].s) + f2d_bits(tot[c].c);
            b.aacc.c[c][g] = f2d_bits(tot[3 + c].s) + f2d_bits(tot[3 + c].c);
        }
    }
}

__global__ void __launch_bounds__(32 * kTileWarps) batch_mixed_tiles_kernel(const __grid_constant__ Batch b,
                                                                           int first_step, int nsteps, int skip,
                                                                           int do_init)
{
    __shared__ TileSmem ts;
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
            const double pe = tile_pass_mixed<true>(b, off, n, M, kin, kout, ts);
            __syncthreads();
            tile_totals(b, off, n);
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
                pe = tile_pass_mixed<true>(b, off, n, M, kin, kout, ts);
            else
                tile_pass_mixed<false>(b, off, n, M, kin, kout, ts);
            __syncthreads();
            tile_totals(b, off, n);
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
        case 0: batch_mixed_tiles_kernel<<<blocks, threads, 0, st>>>(b, first_step, nsteps, skip, do_init); break;
        case 32: batch_mixed_kernel<32><<<blocks, threads, 0, st>>>(b, first_step, nsteps, skip, do_init); break;
        case 64: batch_mixed_kernel<64><<<blocks, threads, 0, st>>>(b, first_step, nsteps, skip, do_init); break;
        default: batch_mixed_kernel<128><<<blocks, threads, 0, st>>>(b, first_step, nsteps, skip, do_init); break;
    }
}

int batch_mixed_max_blocks_per_sm(int tile, int threads)
{
    int nb = 0;
    switch (tile) {
        case 0: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, batch_mixed_tiles_kernel, threads, 0); break;
        case 32: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, batch_mixed_kernel<32>, threads, 0); break;
        case 64: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, batch_mixed_kernel<64>, threads, 0); break;
        default: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, batch_mixed_kernel<128>, threads, 0); break;
    }
    return nb;
}

}  // namespace sl
