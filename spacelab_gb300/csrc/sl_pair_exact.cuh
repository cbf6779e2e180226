// sl_pair_exact.cuh -- FP64 pair physics of the reference's pass 2 in the
// reference's operation order (ColliderSingleCore.cpp:104-253, vec3.hpp
// semantics).  Shared by the all-pairs tile kernel and the batched solver;
// every file that includes it is compiled with --fmad=false.
#pragma once
#include "sl_device.cuh"
#include "sl_fp64_exact.cuh"

namespace sl {

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

// vdw_coef with the quotient rounded from an integer-pipe reciprocal
// estimate (sl_fp64_exact.cuh): the same IEEE result.
__device__ __forceinline__ double vdw_coef_fix(double h, double Ra, double Rb, double twoRa, double twoRb,
                                               double fourRa, double cR3a)
{
    const double h2 = h * h;
    const double S = h2 + twoRa * h + twoRb * h;
    const double T = S + fourRa * Rb;
    const double den = S * S * T * T;
    return cR3a * Rb * Rb * Rb * div_by_fixed<true>(h + Ra + Rb, den, recip_newton(den));
}

// vdw_coef_fix for a pair of equal radii R (Ra == Rb bit for bit), with the
// pair-independent products hoisted: c4 = fourR * R and
// P = ((cR3 * R) * R) * R.  Every remaining operation is the general
// form's, in its order, so the result is the same bits.
__device__ __forceinline__ double vdw_coef_uniform(double h, double R, double twoR, double c4, double P)
{
    const double h2 = h * h;
    const double t = twoR * h;      // twoRa * h == twoRb * h
    const double S = h2 + t + t;
    const double T = S + c4;
    const double den = S * S * T * T;
    return P * div_by_fixed<true>(h + R + R, den, recip_newton(den));
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
// A > B, rVecab = pos[B] - pos[A].
template <bool WRITE>
__device__ __noinline__ ContactOut contact_pair_exact(const ContactIn& in, const Material& M, double rx, double ry,
                                                      double rz, double dist, double overlap, double Ra,
                                                      double Rb, double twoRa, double twoRb, double fourRa,
                                                      double cR3a)
{
    const double sumRaRb = Ra + Rb;
    // k from the previous-step distance (:119-126), recomputed from the
    // previous positions with the same operation sequence as `dist`.
    const double px = in.prevB[0] - in.prevA[0];
    const double py = in.prevB[1] - in.prevA[1];
    const double pz = in.prevB[2] - in.prevA[2];
    const double oldDist = sqrt(px * px + py * py + pz * pz);
    const double k = (dist >= oldDist) ? in.kout : in.kin;

    const double h = M.h_min;
    const double coef = vdw_coef(h, Ra, Rb, twoRa, twoRb, fourRa, cR3a);
    const double nx = rx / dist, ny = ry / dist, nz = rz / dist;  // normalized() == rVecab/dist
    const double vdwx = coef * nx, vdwy = coef * ny, vdwz = coef * nz;
    const double es = -k * overlap * .5;                          // :142
    const double ex = es * nx, ey = es * ny, ez = es * nz;
    const double gs = M.G * in.mA * in.mB / (dist * dist);      // :145
    const double gx = gs * nx, gy = gs * ny, gz = gs * nz;

    const double efm = sqrt(ex * ex + ey * ey + ez * ez);         // :154
    const double rax = (rx * Ra) / sumRaRb, ray = (ry * Ra) / sumRaRb, raz = (rz * Ra) / sumRaRb;
    const double rbx = (-rx * Rb) / sumRaRb, rby = (-ry * Rb) / sumRaRb, rbz = (-rz * Rb) / sumRaRb;
    const double wax = in.wA[0], way = in.wA[1], waz = in.wA[2];
    const double wbx = in.wB[0], wby = in.wB[1], wbz = in.wB[2];
    const double wdx = wax - wbx, wdy = way - wby, wdz = waz - wbz;  // :157
    const double dvx = in.vB[0] - in.vA[0];                         // :160
    const double dvy = in.vB[1] - in.vA[1];
    const double dvz = in.vB[2] - in.vA[2];
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

}  // namespace sl
