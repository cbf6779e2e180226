// sl_step.cu -- the FP64 step of SpaceLab's hot path on sm_103a, bit-exact
// with the reference's sim_one_step (ColliderSingleCore.cpp:78-288).
//
// One step is four launches on the handle's stream:
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
// no multiply-add is contracted; fma() appears only in div_by_recip.
#include "sl_device.cuh"
#include "sl_kernels.h"

#include <cstdio>

namespace sl {

// ---------------------------------------------------------------- pass 1 --
__global__ void __launch_bounds__(256) drift_kernel(const __grid_constant__ System s)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= s.n) return;
    const double dt = s.sc->dt;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const double vh = s.vel.c[c][i] + (.5 * s.acc.c[c][i]) * dt;   // :84
        const double whc = s.w.c[c][i] + (.5 * s.aacc.c[c][i]) * dt;   // :87
        const double p = s.pos.c[c][i];
        s.velh.c[c][i] = vh;
        s.wh.c[c][i] = whc;
        s.prev.c[c][i] = p;            // positions the pair distances of
        s.pos.c[c][i] = p + vh * dt;   // the previous step were taken at; :90
    }
}

// ---------------------------------------------------------------- pass 2 --
// Per-warp staging of the A block (lane l holds sphere X*32+l).
struct ABlock {
    double x[kBlock], y[kBlock], z[kBlock], R[kBlock], twoR[kBlock], fourR[kBlock], cR3[kBlock],
        m[kBlock], inv_m[kBlock];
};

// vdW force magnitude prefix chain of ColliderSingleCore.cpp:135-139 /
// :221-225:  Ha/6*64*Ra*Ra*Ra*Rb*Rb*Rb * ((h+Ra+Rb) / (S*S*T*T)),
// S = h2 + 2Ra h + 2Rb h, T = S + 4 Ra Rb; cR3 = ((Ha/6*64)*Ra)*Ra*Ra.
__device__ __forceinline__ double vdw_coef(double h, double Ra, double Rb, double twoRa, double twoRb,
                                           double fourRa, double cR3a)
{
    const double h2 = h * h;
    const double S = h2 + twoRa * h + twoRb * h;
    const double T = S + fourRa * Rb;
    return cR3a * Rb * Rb * Rb * ((h + Ra + Rb) / (S * S * T * T));
}

// U_vdw of ColliderSingleCore.cpp:195-202 / :231-238.
__device__ __forceinline__ double vdw_energy(double Ha, double h, double Ra, double Rb, double twoRa)
{
    const double sumRaRb = Ra + Rb;
    const double diffRaRb = Ra - Rb;
    const double z = sumRaRb + h;
    const double two_RaRb = twoRa * Rb;
    const double denom_sum = z * z - (sumRaRb * sumRaRb);
    const double denom_diff = z * z - (diffRaRb * diffRaRb);
    return -Ha / 6 * (two_RaRb / denom_sum + two_RaRb / denom_diff + log(denom_sum / denom_diff));
}

struct ContactOut {
    double fx, fy, fz;      // totalForceOnA
    double tax, tay, taz;   // torqueA
    double tbx, tby, tbz;   // torqueB
    double pe;
};

// Contact branch, ColliderSingleCore.cpp:119-204, for the pair (A, B),
// A > B, rVecab = pos[B] - pos[A].  Rare (O(N) of the O(N^2) pairs), so its
// operands beyond positions and radii are fetched here from global memory.
template <bool WRITE>
__device__ __noinline__ ContactOut contact_pair(const System& s, int A, int B, double rx, double ry,
                                                double rz, double dist, double overlap, double Ra,
                                                double Rb, double twoRa, double twoRb, double fourRa,
                                                double cR3a)
{
    const Material& M = s.mat;
    const double sumRaRb = Ra + Rb;
    // k from the previous-step distance (:119-126), recomputed from the
    // previous positions with the same operation sequence as `dist`.
    const double px = s.prev.c[0][B] - s.prev.c[0][A];
    const double py = s.prev.c[1][B] - s.prev.c[1][A];
    const double pz = s.prev.c[2][B] - s.prev.c[2][A];
    const double oldDist = sqrt(px * px + py * py + pz * pz);
    const double k = (dist >= oldDist) ? s.sc->kout : s.sc->kin;

    const double h = M.h_min;
    const double coef = vdw_coef(h, Ra, Rb, twoRa, twoRb, fourRa, cR3a);
    const double nx = rx / dist, ny = ry / dist, nz = rz / dist;  // normalized() == rVecab/dist
    const double vdwx = coef * nx, vdwy = coef * ny, vdwz = coef * nz;
    const double es = -k * overlap * .5;                          // :142
    const double ex = es * nx, ey = es * ny, ez = es * nz;
    const double gs = M.G * s.m[A] * s.m[B] / (dist * dist);      // :145
    const double gx = gs * nx, gy = gs * ny, gz = gs * nz;

    const double efm = sqrt(ex * ex + ey * ey + ez * ez);         // :154
    const double rax = (rx * Ra) / sumRaRb, ray = (ry * Ra) / sumRaRb, raz = (rz * Ra) / sumRaRb;
    const double rbx = (-rx * Rb) / sumRaRb, rby = (-ry * Rb) / sumRaRb, rbz = (-rz * Rb) / sumRaRb;
    const double wax = s.w.c[0][A], way = s.w.c[1][A], waz = s.w.c[2][A];
    const double wbx = s.w.c[0][B], wby = s.w.c[1][B], wbz = s.w.c[2][B];
    const double wdx = wax - wbx, wdy = way - wby, wdz = waz - wbz;  // :157
    const double dvx = s.vel.c[0][B] - s.vel.c[0][A];               // :160
    const double dvy = s.vel.c[1][B] - s.vel.c[1][A];
    const double dvz = s.vel.c[2][B] - s.vel.c[2][A];
    // frame_A_vel_B, :161-162
    const double dot = dvx * rx + dvy * ry + dvz * rz;
    const double dd = dist * dist;
    const double ux = rx / dd, uy = ry / dd, uz = rz / dd;
    const double cax = way * raz - waz * ray, cay = waz * rax - wax * raz, caz = wax * ray - way * rax;
    const double cbx = wby * raz - wbz * ray, cby = wbz * rax - wbx * raz, cbz = wbx * ray - wby * rax;
    const double fvx = dvx - dot * ux - cax - cbx;
    const double fvy = dvy - dot * uy - cay - cby;
    const double fvz = dvz - dot * uz - caz - cbz;

    double sx = 0, sy = 0, sz = 0;
    const double rvm = sqrt(fvx * fvx + fvy * fvy + fvz * fvz);
    if (rvm > 1e-13) {                                            // :166-170
        const double ss = M.u_s * efm;
        sx = ss * (fvx / rvm); sy = ss * (fvy / rvm); sz = ss * (fvz / rvm);
    }
    double qx = 0, qy = 0, qz = 0;
    const double wdm = sqrt(wdx * wdx + wdy * wdy + wdz * wdz);
    if (wdm > 1e-13) {                                            // :174-178
        const double cx = wdy * raz - wdz * ray, cy = wdz * rax - wdx * raz, cz = wdx * ray - wdy * rax;
        const double cn = sqrt(cx * cx + cy * cy + cz * cz);
        const double rs = -M.u_r * efm;
        qx = (rs * cx) / cn; qy = (rs * cy) / cn; qz = (rs * cz) / cn;
    }
    ContactOut o;
    o.fx = gx + ex + sx + vdwx;                                   // :181
    o.fy = gy + ey + sy + vdwy;
    o.fz = gz + ez + sz + vdwz;
    const double pax = sx + qx, pay = sy + qy, paz = sz + qz;     // :184
    o.tax = ray * paz - raz * pay; o.tay = raz * pax - rax * paz; o.taz = rax * pay - ray * pax;
    const double pbx = -sx + qx, pby = -sy + qy, pbz = -sz + qz;  // :185
    o.tbx = rby * pbz - rbz * pby; o.tby = rbz * pbx - rbx * pbz; o.tbz = rbx * pby - rby * pbx;
    o.pe = 0;
    if (WRITE) o.pe = vdw_energy(M.Ha, h, Ra, Rb, twoRa) + 0.5 * k * overlap * overlap;  // :203
    return o;
}

// One warp per lower-triangular 32x32 block tile (X, Y), X >= Y.  Lane b
// owns sphere B = 32Y + b and walks the 32 spheres A = 32X + a of the A
// block; on the diagonal only a > b is a pair.  Tiles are independent, so
// the grid is a static stride over all tiles.
template <bool WRITE>
__global__ void __launch_bounds__(128, 2) pair_tile_kernel(const __grid_constant__ System s)
{
    __shared__ ABlock sA[4];
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    ABlock& ab = sA[wib];
    const long long nwarps = (long long)gridDim.x * 4;
    const size_t plane = (size_t)s.npad * s.npad;
    const double Ha = s.mat.Ha, h_min = s.mat.h_min;

    for (long long t = (long long)blockIdx.x * 4 + wib; t < s.ntiles; t += nwarps) {
        int X, Y;
        tile_coords(t, X, Y);
        {
            const int i = X * kBlock + lane;  // < npad always
            ab.x[lane] = s.pos.c[0][i]; ab.y[lane] = s.pos.c[1][i]; ab.z[lane] = s.pos.c[2][i];
            ab.R[lane] = s.R[i]; ab.twoR[lane] = s.twoR[i]; ab.fourR[lane] = s.fourR[i];
            ab.cR3[lane] = s.cR3[i]; ab.m[lane] = s.m[i]; ab.inv_m[lane] = s.inv_m[i];
        }
        __syncwarp();
        const int B = Y * kBlock + lane;
        const bool bvalid = B < s.n;
        const double bx = s.pos.c[0][B], by = s.pos.c[1][B], bz = s.pos.c[2][B];
        const double Rb = s.R[B], twoRb = s.twoR[B], mb = s.m[B], inv_mb = s.inv_m[B];
        const int a_end = min(kBlock, s.n - X * kBlock);
        double pe = 0;
        uint32_t rowbits = 0, colbits = 0;
        double* rowA = s.pairbuf + (size_t)(X * kBlock) * s.npad + B;  // + a*npad: term for A
        double* rowB = s.pairbuf + (size_t)B * s.npad + X * kBlock;    // + a: term for B

        for (int a = 0; a < a_end; ++a) {
            const bool valid = bvalid && (X != Y || lane < a);
            bool contact = false;
            if (valid) {
                const int A = X * kBlock + a;
                const double Ra = ab.R[a];
                const double sumRaRb = Ra + Rb;                              // :104
                const double rx = bx - ab.x[a], ry = by - ab.y[a], rz = bz - ab.z[a];  // :105
                const double dist = sqrt(rx * rx + ry * ry + rz * rz);      // :107
                const double overlap = sumRaRb - dist;                        // :110
                double fx, fy, fz;
                if (overlap > 0) {
                    contact = true;
                    const ContactOut o = contact_pair<WRITE>(s, A, B, rx, ry, rz, dist, overlap, Ra, Rb,
                                                             ab.twoR[a], twoRb, ab.fourR[a], ab.cR3[a]);
                    fx = o.fx; fy = o.fy; fz = o.fz;
                    const double im_a = s.inv_moi[A], mo_a = s.moi[A];
                    const double im_b = s.inv_moi[B], mo_b = s.moi[B];
                    double* ta = s.torqbuf + (size_t)A * s.npad + B;   // :187
                    double* tb = s.torqbuf + (size_t)B * s.npad + A;   // :188
                    ta[0] = div_by_recip(o.tax, mo_a, im_a);
                    ta[plane] = div_by_recip(o.tay, mo_a, im_a);
                    ta[2 * plane] = div_by_recip(o.taz, mo_a, im_a);
                    tb[0] = div_by_recip(o.tbx, mo_b, im_b);
                    tb[plane] = div_by_recip(o.tby, mo_b, im_b);
                    tb[2 * plane] = div_by_recip(o.tbz, mo_b, im_b);
                    if (WRITE) pe += o.pe;
                } else {
                    double h = fabs(overlap);                                  // :211-215
                    if (h < h_min) h = h_min;
                    const double coef = vdw_coef(h, Ra, Rb, ab.twoR[a], twoRb, ab.fourR[a], ab.cR3[a]);
                    fx = coef * (rx / dist); fy = coef * (ry / dist); fz = coef * (rz / dist);  // :221-227
                    if (WRITE) pe += vdw_energy(Ha, h, Ra, Rb, ab.twoR[a]);                    // :239
                }
                // :249-250 -- acc[A] += F/m[A]; acc[B] -= F/m[B] (stored negated)
                const double ma = ab.m[a], ima = ab.inv_m[a];
                double* pa = rowA + (size_t)a * s.npad;
                __stcs(pa, div_by_recip(fx, ma, ima));
                __stcs(pa + plane, div_by_recip(fy, ma, ima));
                __stcs(pa + 2 * plane, div_by_recip(fz, ma, ima));
                double* pb = rowB + a;
                __stcs(pb, -div_by_recip(fx, mb, inv_mb));
                __stcs(pb + plane, -div_by_recip(fy, mb, inv_mb));
                __stcs(pb + 2 * plane, -div_by_recip(fz, mb, inv_mb));
            }
            const uint32_t bal = __ballot_sync(0xffffffffu, contact);
            if (lane == a) rowbits = bal;
            if (contact) colbits |= 1u << a;
        }
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
    }
}

// ------------------------------------------------- row sums + pass 3 ------
// Thread (c, i): acc_c[i] = sum over partners j ascending of pairbuf[c][i][j]
// (j != i), aacc_c[i] likewise over the contact partners, then pass 3.
// The sum is a dependent chain per (c, i), so the kernel is latency-bound:
// each thread keeps kRowBatch 16-byte loads of its row in flight (register
// double buffering) while it adds the previous batch.
constexpr int kRowBatch = 16;
constexpr int kRowThreads = 32;

__global__ void __launch_bounds__(kRowThreads) rowsum_kernel(const __grid_constant__ System s)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 3 * s.n) return;
    const int c = t / s.n;
    const int i = t - c * s.n;
    const int n = s.n;
    const size_t plane = (size_t)s.npad * s.npad;
    const double2* row = reinterpret_cast<const double2*>(s.pairbuf + c * plane + (size_t)i * s.npad);
    const int nv = (n + 1) / 2;  // double2 words covering columns [0, n)
    double2 cur[kRowBatch], nxt[kRowBatch];
#pragma unroll
    for (int k = 0; k < kRowBatch; ++k) cur[k] = k < nv ? __ldcs(row + k) : make_double2(0.0, 0.0);
    double acc = 0.0;
    for (int base = 0; base < nv; base += kRowBatch) {
#pragma unroll
        for (int k = 0; k < kRowBatch; ++k) {
            const int q = base + kRowBatch + k;
            nxt[k] = q < nv ? __ldcs(row + q) : make_double2(0.0, 0.0);
        }
#pragma unroll
        for (int k = 0; k < kRowBatch; ++k) {
            const int j = 2 * (base + k);
            if (j < n && j != i) acc += cur[k].x;
            if (j + 1 < n && j + 1 != i) acc += cur[k].y;
        }
#pragma unroll
        for (int k = 0; k < kRowBatch; ++k) cur[k] = nxt[k];
    }
    double aacc = 0.0;
    const uint32_t* mrow = s.cmask + (size_t)i * s.nb;
    const double* trow = s.torqbuf + c * plane + (size_t)i * s.npad;
    for (int Y = 0; Y < s.nb; ++Y) {
        uint32_t wd = mrow[Y];
        while (wd) {
            const int b = __ffs(wd) - 1;
            wd &= wd - 1;
            aacc += trow[Y * kBlock + b];
        }
    }
    const double dt = s.sc->dt;
    const double v = s.velh.c[c][i] + (.5 * acc) * dt;    // :265
    const double wv = s.wh.c[c][i] + (.5 * aacc) * dt;    // :266
    s.acc.c[c][i] = acc;
    s.aacc.c[c][i] = aacc;
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
    for (long long t = tid; t < s.ntiles; t += kRedThreads) v[0] += s.pe_tile[t];
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
    s.inv_m[i] = 1.0 / m;
    s.inv_moi[i] = 1.0 / moi;
}

// ------------------------------------------------------------ launchers --
int pair_grid_blocks(const System& s, int num_sms)
{
    long long want = (s.ntiles + 3) / 4;
    long long cap = (long long)num_sms * 2;  // 2 CTAs (8 warps) per SM
    return (int)(want < cap ? want : cap);
}

void launch_derive(const System& s, cudaStream_t st)
{
    derive_kernel<<<(s.npad + 255) / 256, 256, 0, st>>>(s);
}

void launch_step(const System& s, bool write, int num_sms, cudaStream_t st, StepTimers* tm)
{
    drift_kernel<<<(s.n + 255) / 256, 256, 0, st>>>(s);
    if (tm) cudaEventRecord(tm->ev[0], st);
    const int pb = pair_grid_blocks(s, num_sms);
    if (write)
        pair_tile_kernel<true><<<pb, 128, 0, st>>>(s);
    else
        pair_tile_kernel<false><<<pb, 128, 0, st>>>(s);
    if (tm) cudaEventRecord(tm->ev[1], st);
    rowsum_kernel<<<(3 * s.n + kRowThreads - 1) / kRowThreads, kRowThreads, 0, st>>>(s);
    if (tm) cudaEventRecord(tm->ev[2], st);
    if (write) {
        const int nred = kRedBlocks;
        const int chunk = (s.n + nred - 1) / nred;
        energy_partial_kernel<<<nred, kRedThreads, 0, st>>>(s, chunk);
        energy_final_kernel<<<1, kRedThreads, 0, st>>>(s, nred);
    }
}

}  // namespace sl
