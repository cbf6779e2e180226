// sl_pair_mixed.cuh -- pair physics of the mixed-precision form: FP32
// forces and torques on FP64 displacements and squared gaps, FP64 write-step
// potential energy (ColliderSingleCore.cpp:104-253 term by term).  Shared by
// the all-pairs mixed kernels and the batched mixed solver.
#pragma once
#include "sl_device.cuh"

namespace sl {

// vdW magnitude in scaled lengths: Ra^3 Rb^3 (h+Ra+Rb) / (S^2 T^2) with
// S = h^2 + 2Ra h + 2Rb h and T = S + 4 Ra Rb (ColliderSingleCore.cpp:135-139).
// Times Ha/6*64 / L it is the force in dyn.
__device__ __forceinline__ float vdw_shape(float h, float Ra, float Rb)
{
    const float sum = Ra + Rb;
    const float S = h * (h + 2.0f * sum);
    const float T = S + 4.0f * Ra * Rb;
    const float r3 = (Ra * Ra * Ra) * (Rb * Rb * Rb);
    // fast FP32 quotient (MUFU reciprocal, ~2 ulp): the denominator stays
    // far below 2^126 for separations up to ~10^4 radii
    return __fdividef(r3 * (h + sum), (S * S) * (T * T));
}

// Pairs with |r|^2 >= far_sq (R_A + R_B)^2 take the FP32 vdW path without a
// square root.  far = max(1.25, 1 + h_min / (2 R_min)): their gap
// h = |r| - R_A - R_B is then at least (R_A + R_B) / 4 and above the clamp
// h_min, so S = |r|^2 - (R_A + R_B)^2 = h (h + 2 (R_A + R_B)) keeps all but
// ~1.5 bits of |r|^2's precision, and the force comes out within ~2e-6 of the
// FP64 formula (measured over separations 1.25-4 radii sums, split positions
// up to 60 radii from the origin).  Closer pairs -- contacts and small gaps --
// take the double-float geometry.  The far pairs' write-step potential is
// the series of vdw_bracket, valid over the same range.
inline float far_threshold_sq(double h_min, double r_min)
{
    double far = 1.0 + h_min / (2.0 * r_min);
    if (far < 1.25) far = 1.25;
    return (float)(far * far);
}

// Approximate FP32 reciprocal (one MUFU instruction, relative error below
// 2^-22; subnormal inputs and results flush to zero).
__device__ __forceinline__ float rcp_approx(float x)
{
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// The vdW potential's bracket 2RaRb/P + 2RaRb/Q + ln(P/Q), P = z^2 - (Ra+Rb)^2,
// Q = z^2 - (Ra-Rb)^2 (ColliderSingleCore.cpp:228-240; U = -Ha/6 times it),
// for a pair at centre distance z >= far (Ra + Rb), from d2 = z^2 in scaled
// lengths.  Its O(z^-2) and O(z^-4) parts cancel exactly, which the closed
// form resolves only in FP64.  With w = 2 Ra Rb / (z^2 - Ra^2 - Rb^2)
// (u = 4 Ra Rb / Q = 2w / (1 + w), so 1 - u = (1 - w) / (1 + w)) the bracket
// is 2w/(1 - w^2) - 2 atanh(w) = sum_{j>=1} 4j/(2j+1) w^(2j+1), all terms
// positive.  At z >= 1.25 (Ra + Rb), w <= 0.47 and w^2 <= 0.22: twelve
// terms by Horner in FP32 leave a relative truncation error below 2e-8
// (checked against 40-digit arithmetic); the FP32 rounding of z^2 bounds the
// result to ~7e-7 relative.
__device__ __forceinline__ float vdw_bracket(float d2, float Ra, float Rb)
{
    const float w = (2.0f * Ra * Rb) * rcp_approx(fmaf(-Ra, Ra, fmaf(-Rb, Rb, d2)));
    const float x = w * w;
    float p = 48.0f / 25.0f;                 // j = 12: 4j/(2j+1)
    p = fmaf(p, x, 44.0f / 23.0f);           // 11
    p = fmaf(p, x, 40.0f / 21.0f);           // 10
    p = fmaf(p, x, 36.0f / 19.0f);           // 9
    p = fmaf(p, x, 32.0f / 17.0f);           // 8
    p = fmaf(p, x, 28.0f / 15.0f);           // 7
    p = fmaf(p, x, 24.0f / 13.0f);           // 6
    p = fmaf(p, x, 20.0f / 11.0f);           // 5
    p = fmaf(p, x, 16.0f / 9.0f);            // 4
    p = fmaf(p, x, 12.0f / 7.0f);            // 3
    p = fmaf(p, x, 8.0f / 5.0f);             // 2
    p = fmaf(p, x, 4.0f / 3.0f);             // 1
    return (w * x) * p;
}

struct ContactF {
    float fx, fy, fz, tax, tay, taz, tbx, tby, tbz;
    double k;  // spring constant chosen for this step (for the write-step PE)
};

// Write-step potential energy of one pair in FP64 (energy sums are FP64;
// the vdW bracket cancels to O(R^6/z^6) from O(R^2/z^2) terms for distant
// pairs, which FP32 cannot resolve): U_vdw, plus 0.5 k overlap^2 in contact
// (ColliderSingleCore.cpp:190-204, 228-240).  overlap = g / (R_A+R_B+|r|).
__device__ __forceinline__ double pair_pe_fp64(const Material& M, double Ra, double Rb, double gap2, double d2,
                                               bool contact, double k)
{
    const double sum = Ra + Rb;
    const double overlap = gap2 / (sum + sqrt(d2));
    const double h = contact ? M.h_min : fmax(-overlap, M.h_min);
    const double diff = Ra - Rb;
    const double z = sum + h;
    const double two = 2 * Ra * Rb;
    const double ds = h * (2 * sum + h);
    const double dd = (z - diff) * (z + diff);
    double U = -M.Ha / 6 * (two / ds + two / dd + log(ds / dd));
    if (contact) U += 0.5 * k * overlap * overlap;
    return U;
}

// Contact branch (ColliderSingleCore.cpp:119-204) in FP32, physical units
// except where noted.  nx,ny,nz: unit vector A->B; dist, overlap in cm;
// Ras, Rbs radii scaled by 2^-len_shift.
static __device__ __noinline__ ContactF contact_mixed(const ContactIn& in, const Material& M, int len_shift, double d2,
                                               float nx, float ny, float nz, float dist, float overlap, float Ras,
                                               float Rbs)
{
    // kin/kout from the previous-step distance, compared in FP64 on |r|^2
    const double px = in.prevB[0] - in.prevA[0];
    const double py = in.prevB[1] - in.prevA[1];
    const double pz = in.prevB[2] - in.prevA[2];
    const double d2_old = fma(px, px, fma(py, py, pz * pz));
    const double kd = (d2 >= d2_old) ? in.kout : in.kin;
    const float k = (float)kd;

    const float L = ldexpf(1.0f, len_shift);
    const float hs = (float)M.h_min / L;
    const float vdw = (float)(M.Ha / 6 * 64) / L * vdw_shape(hs, Ras, Rbs);
    const float es = -k * overlap * 0.5f;                                     // :142
    const float gs = (float)M.G * (float)in.mA * (float)in.mB / (dist * dist);  // :145
    const float efm = fabsf(es);                                               // :154
    const float Ra = Ras * L, Rb = Rbs * L, sum = Ra + Rb;
    const float rax = nx * dist * Ra / sum, ray = ny * dist * Ra / sum, raz = nz * dist * Ra / sum;  // :155
    const float rbx = -nx * dist * Rb / sum, rby = -ny * dist * Rb / sum, rbz = -nz * dist * Rb / sum;
    const float wax = (float)in.wA[0], way = (float)in.wA[1], waz = (float)in.wA[2];
    const float wbx = (float)in.wB[0], wby = (float)in.wB[1], wbz = (float)in.wB[2];
    const float wdx = wax - wbx, wdy = way - wby, wdz = waz - wbz;            // :157
    const float dvx = (float)(in.vB[0] - in.vA[0]);                           // :160
    const float dvy = (float)(in.vB[1] - in.vA[1]);
    const float dvz = (float)(in.vB[2] - in.vA[2]);
    const float dn = dvx * nx + dvy * ny + dvz * nz;                          // :161-162
    const float fvx = dvx - dn * nx - (way * raz - waz * ray) - (wby * raz - wbz * ray);
    const float fvy = dvy - dn * ny - (waz * rax - wax * raz) - (wbz * rax - wbx * raz);
    const float fvz = dvz - dn * nz - (wax * ray - way * rax) - (wbx * ray - wby * rax);
    float sx = 0, sy = 0, sz = 0;
    const float rvm = sqrtf(fvx * fvx + fvy * fvy + fvz * fvz);
    if (rvm > 1e-13f) {                                                       // :166-170
        const float f = M.u_s * efm / rvm;
        sx = f * fvx; sy = f * fvy; sz = f * fvz;
    }
    float qx = 0, qy = 0, qz = 0;
    const float wdm = sqrtf(wdx * wdx + wdy * wdy + wdz * wdz);
    if (wdm > 1e-13f) {                                                       // :174-178
        const float cx = wdy * raz - wdz * ray, cy = wdz * rax - wdx * raz, cz = wdx * ray - wdy * rax;
        const float cn = sqrtf(cx * cx + cy * cy + cz * cz);
        if (cn > 0.0f) {
            const float f = -(float)M.u_r * efm / cn;
            qx = f * cx; qy = f * cy; qz = f * cz;
        }
    }
    const float fn = gs + es + vdw;                                           // :181 (radial parts)
    ContactF o;
    o.fx = fn * nx + sx; o.fy = fn * ny + sy; o.fz = fn * nz + sz;
    const float pax = sx + qx, pay = sy + qy, paz = sz + qz;                  // :184
    o.tax = ray * paz - raz * pay; o.tay = raz * pax - rax * paz; o.taz = rax * pay - ray * pax;
    const float pbx = -sx + qx, pby = -sy + qy, pbz = -sz + qz;               // :185
    o.tbx = rby * pbz - rbz * pby; o.tby = rbz * pbx - rbx * pbz; o.tbz = rbx * pby - rby * pbx;
    o.k = kd;
    return o;
}

}  // namespace sl
