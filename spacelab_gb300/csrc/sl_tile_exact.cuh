// sl_tile_exact.cuh -- the exact form's pairs of one 32 x 32 block tile
// (ColliderSingleCore.cpp:104-253 for each pair, in the reference's
// orientation A > B), shared by the single-system pair kernel (sl_step.cu)
// and the batched exact solver's pair-tile pass (sl_batch.cu).  Must be
// compiled with --fmad=false (the exact arithmetic contract).
#pragma once
#include "sl_device.cuh"
#include "sl_fp64_exact.cuh"
#include "sl_pair_exact.cuh"
#include "sl_vdw_energy.cuh"

namespace sl {

// Per-warp staging of the A block (lane l holds sphere X*32+l).
struct ABlock {
    double x[kBlock], y[kBlock], z[kBlock], R[kBlock], twoR[kBlock], fourR[kBlock], cR3[kBlock], m[kBlock];
    unsigned long long rm[kBlock];
};

// Equal radii across a tile (monodisperse clusters): the sum of radii and
// the vdW coefficient's radius products are the same for every pair of the
// tile and are formed once (vdw_coef_uniform).
struct TileUniform {
    double R0, twoR0, sum0, c40, P0;
};

// Per-warp shared staging of sphere B's terms (lane = B) for four
// consecutive partners: [component][lane][4 + 1 padding] doubles, so that a
// lane's 8-byte accesses at a 40-byte stride fall in distinct banks per
// half-warp.
constexpr int kBStageRow = 5;
constexpr int kBStagePlane = kBlock * kBStageRow;
constexpr int kBStageDoubles = 3 * kBStagePlane;

// The pairs of one tile (X, Y) for lane = sphere B: terms to pairbuf and
// torqbuf, contact bits to rowbits/colbits, PE (write steps) to pe.
// bstage (kBStageDoubles per warp, or NULL): off the diagonal, sphere B's
// terms -- which go to B's own row of pairbuf, a different row per lane --
// are gathered four at a time and written as whole 32-byte sectors (two
// 16-byte stores per component) instead of one 8-byte store per term from
// 32 rows at once; partners past the last sphere are written as +0.0, the
// value those entries hold anyway.  On the diagonal tile, and with NULL,
// every term is stored as it is computed.
template <bool WRITE, bool UNI>
__device__ __forceinline__ void tile_pairs(const System& s, const ABlock& ab, int X, int Y, int lane, int a_end,
                                           double bx, double by, double bz, double Rb, double twoRb, double mb,
                                           unsigned long long rmb, bool bvalid, const TileUniform& tu,
                                           long long h_min_bits, double Ha, double* rowA, double* rowB,
                                           double& pe, uint32_t& rowbits, uint32_t& colbits,
                                           double* bstage = nullptr)
{
    const size_t plane = (size_t)s.npad * s.npad;
    const int B = Y * kBlock + lane;
    const bool staged = bstage != nullptr && X != Y;
    double* my_stage = staged ? bstage + lane * kBStageRow : nullptr;
    for (int a = 0; a < a_end; ++a) {
        const bool valid = bvalid && (X != Y || lane < a);
        bool contact = false;
        if (valid) {
            const int A = X * kBlock + a;
            const double Ra = ab.R[a];
            const double sumRaRb = UNI ? tu.sum0 : Ra + Rb;              // :104
            const double rx = bx - ab.x[a], ry = by - ab.y[a], rz = bz - ab.z[a];  // :105
            const double d2 = rx * rx + ry * ry + rz * rz;
            int p;
            unsigned long long F;
            const unsigned long long Yr = rsqrt_fix(d2, p, F);            // ~1/sqrt(d2), integer pipe
            const double dist = sqrt_fix(d2, F, Yr, p);                   // :107, RN(sqrt)
            const double overlap = sumRaRb - dist;                        // :110
            // the comparisons of the step are made on the bit patterns
            // (integer pipe): for doubles of one sign the integer order
            // is the FP order; NaN is excluded explicitly
            const long long ob = __double_as_longlong(overlap);
            double fx, fy, fz;
            if (ob > 0 && ob <= 0x7ff0000000000000ll) {                    // overlap > 0
                contact = true;
                const ContactIn in = gather_contact(s, A, B);
                const ContactOut o = contact_pair_exact<WRITE>(in, s.mat, rx, ry, rz, dist, overlap, Ra, Rb,
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
                long long hb = ob & 0x7fffffffffffffffll;                  // :211-215 |overlap|
                if (hb < h_min_bits) hb = h_min_bits;                      // h < h_min (NaN stays NaN)
                const double h = __longlong_as_double(hb);
                const double coef = UNI ? vdw_coef_uniform(h, tu.R0, tu.twoR0, tu.c40, tu.P0)
                                        : vdw_coef_fix(h, Ra, Rb, ab.twoR[a], twoRb, ab.fourR[a], ab.cR3[a]);
                fx = coef * div_by_rsqrt(rx, dist, Yr, p);                    // :221-227
                fy = coef * div_by_rsqrt(ry, dist, Yr, p);
                fz = coef * div_by_rsqrt(rz, dist, Yr, p);
                if (WRITE) pe += vdw_energy_far_df(Ha, h, Ra, Rb, ab.twoR[a]);             // :239
            }
            // :249-250 -- acc[A] += F/m[A]; acc[B] -= F/m[B] (stored negated)
            const double ma = ab.m[a];
            const unsigned long long rma = ab.rm[a];
            double* pa = rowA + (size_t)a * s.npad;
            __stcs(pa, div_by_fixed<false>(fx, ma, rma));
            __stcs(pa + plane, div_by_fixed<false>(fy, ma, rma));
            __stcs(pa + 2 * plane, div_by_fixed<false>(fz, ma, rma));
            // -(F/m[B]), the sign set in the integer result
            const double tbx = div_by_fixed<false, true>(fx, mb, rmb);
            const double tby = div_by_fixed<false, true>(fy, mb, rmb);
            const double tbz = div_by_fixed<false, true>(fz, mb, rmb);
            if (staged) {
                double* st = my_stage + (a & 3);
                st[0] = tbx;
                st[kBStagePlane] = tby;
                st[2 * kBStagePlane] = tbz;
            } else {
                double* pb = rowB + a;
                __stcs(pb, tbx);
                __stcs(pb + plane, tby);
                __stcs(pb + 2 * plane, tbz);
            }
        }
        const uint32_t bal = __ballot_sync(0xffffffffu, contact);
        if (lane == a) rowbits = bal;
        if (contact) colbits |= 1u << a;
        if (staged && bvalid && ((a & 3) == 3 || a == a_end - 1)) {
            // row B, partners a0 .. a0+3: a 32-byte aligned sector (npad and
            // 32X are multiples of 4, the buffer is 256-byte aligned)
            const int a0 = a & ~3;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const double* st = my_stage + c * kBStagePlane;
                const double v0 = st[0];
                const double v1 = a0 + 1 < a_end ? st[1] : 0.0;
                const double v2 = a0 + 2 < a_end ? st[2] : 0.0;
                const double v3 = a0 + 3 < a_end ? st[3] : 0.0;
                double2* dst = reinterpret_cast<double2*>(rowB + c * plane + a0);
                __stcs(dst, make_double2(v0, v1));
                __stcs(dst + 1, make_double2(v2, v3));
            }
        }
    }
}

}  // namespace sl
