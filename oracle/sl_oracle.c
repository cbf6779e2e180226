/*
 * sl_oracle.c -- CPU oracle for the SpaceLab step (TEST INFRASTRUCTURE ONLY).
 *
 * A plain-C restatement of the reference's sim_one_step and init_conditions,
 * used solely as the checker (tests, smoke(), bench.py's CPU baseline legs).
 * The GPU product library never links or calls this file.
 *
 * Every arithmetic expression is written in the evaluation order that the
 * reference's vec3 class (vec3.hpp:44-128,180-184) and C++ left-to-right
 * associativity produce, so that with -ffp-contract=off the results are
 * bit-identical to the reference compiled with the same flags:
 *   a - b          componentwise                       vec3.hpp:56
 *   v * s, s * v   (s*x, s*y, s*z)                     vec3.hpp:66,180-184
 *   v / s          (x/s, y/s, z/s)                     vec3.hpp:76
 *   dot            (x*vx + y*vy) + z*vz                vec3.hpp:121
 *   cross          (y*vz - z*vy, z*vx - x*vz, x*vy - y*vx)  vec3.hpp:122-125
 *   norm           sqrt((x*x + y*y) + z*z)             vec3.hpp:126
 *   normalized     v / norm()                          vec3.hpp:128
 * Build: gcc -O2 -ffp-contract=off -fopenmp (see spacelab_gb300/build.py).
 */
#include "sl_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

struct slo_sys {
    int n;
    slo_material mat;
    double dt, kin, kout;
    double *pos, *vel, *velh, *acc, *w, *wh, *aacc; /* AoS xyz, 3n each */
    double *R, *m, *moi;
    double* distances;     /* n(n-1)/2, index A*(A-1)/2+B  (ball_group.hpp:741) */
    double* distances_new; /* scratch for the row-parallel step */
};

typedef struct { double x, y, z; } v3;

static inline v3 v3_at(const double* a, long i) { v3 r = {a[3 * i], a[3 * i + 1], a[3 * i + 2]}; return r; }
static inline v3 v3_sub(v3 a, v3 b) { v3 r = {a.x - b.x, a.y - b.y, a.z - b.z}; return r; }
static inline v3 v3_add(v3 a, v3 b) { v3 r = {a.x + b.x, a.y + b.y, a.z + b.z}; return r; }
static inline v3 v3_neg(v3 a) { v3 r = {-a.x, -a.y, -a.z}; return r; }
static inline v3 v3_scale(v3 a, double s) { v3 r = {s * a.x, s * a.y, s * a.z}; return r; }
static inline v3 v3_div(v3 a, double s) { v3 r = {a.x / s, a.y / s, a.z / s}; return r; }
static inline double v3_dot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline v3 v3_cross(v3 a, v3 b)
{
    v3 r = {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
    return r;
}
static inline double v3_norm(v3 a) { return sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
static inline double v3_norm2(v3 a) { return a.x * a.x + a.y * a.y + a.z * a.z; }

static inline long tri_index(long A, long B) { return A * (A - 1) / 2 + B; }

/* Result of one unordered pair (A > B), ColliderSingleCore.cpp:104-253. */
typedef struct {
    v3 force_on_a;   /* totalForceOnA                                 :112,181,227 */
    v3 torque_a;     /* torqueA  (contact only)                        :184 */
    v3 torque_b;     /* torqueB  (contact only)                        :185 */
    double pe;       /* write-step PE term                             :203,239 */
    double dist;     /* new distances[e]                               :253 */
    int contact;
} pair_out;

static inline pair_out pair_eval(const slo_sys* s, int A, int B, double oldDist, int write)
{
    const slo_material* M = &s->mat;
    pair_out o;
    const double sumRaRb = s->R[A] + s->R[B];
    const v3 rVecab = v3_sub(v3_at(s->pos, B), v3_at(s->pos, A));
    const v3 rVecba = v3_neg(rVecab);
    const double dist = v3_norm(rVecab);
    const double overlap = sumRaRb - dist;
    const double Ra = s->R[A];
    const double Rb = s->R[B];
    o.dist = dist;
    o.pe = 0.0;
    if (overlap > 0) {
        o.contact = 1;
        const double k = (dist >= oldDist) ? s->kout : s->kin; /* :122-126 */
        const double h = M->h_min;                            /* :129 */
        const double h2 = h * h;
        const double twoRah = 2 * Ra * h;
        const double twoRbh = 2 * Rb * h;
        const double S = h2 + twoRah + twoRbh;
        const double T = h2 + twoRah + twoRbh + 4 * Ra * Rb;
        const double coef = M->Ha / 6 * 64 * Ra * Ra * Ra * Rb * Rb * Rb * ((h + Ra + Rb) / (S * S * T * T));
        const v3 nrm = v3_div(rVecab, v3_norm(rVecab));             /* normalized() :139 */
        const v3 vdwForceOnA = v3_scale(nrm, coef);
        const v3 elasticForceOnA = v3_scale(v3_div(rVecab, dist), -k * overlap * .5); /* :142 */
        const v3 gravForceOnA =
            v3_scale(v3_div(rVecab, dist), M->G * s->m[A] * s->m[B] / (dist * dist)); /* :145 */
        v3 slideForceOnA = {0, 0, 0};
        v3 rollForceA = {0, 0, 0};
        const double elastic_force_A_mag = v3_norm(elasticForceOnA); /* :154 */
        const v3 r_a = v3_div(v3_scale(rVecab, Ra), sumRaRb);        /* :155 */
        const v3 r_b = v3_div(v3_scale(rVecba, Rb), sumRaRb);        /* :156 */
        const v3 wA = v3_at(s->w, A), wB = v3_at(s->w, B);
        const v3 w_diff = v3_sub(wA, wB);                            /* :157 */
        const v3 d_vel = v3_sub(v3_at(s->vel, B), v3_at(s->vel, A)); /* :160 */
        const v3 frame_A_vel_B =                                     /* :161-162 */
            v3_sub(v3_sub(v3_sub(d_vel, v3_scale(v3_div(rVecab, dist * dist), v3_dot(d_vel, rVecab))),
                          v3_cross(wA, r_a)),
                   v3_cross(wB, r_a));
        const double rel_vel_mag = v3_norm(frame_A_vel_B);
        if (rel_vel_mag > 1e-13) {                                   /* :166-170 */
            slideForceOnA = v3_scale(v3_div(frame_A_vel_B, rel_vel_mag), M->u_s * elastic_force_A_mag);
        }
        const double w_diff_mag = v3_norm(w_diff);
        if (w_diff_mag > 1e-13) {                                    /* :174-178 */
            const v3 c = v3_cross(w_diff, r_a);
            rollForceA = v3_div(v3_scale(c, -M->u_r * elastic_force_A_mag), v3_norm(c));
        }
        o.force_on_a = v3_add(v3_add(v3_add(gravForceOnA, elasticForceOnA), slideForceOnA), vdwForceOnA); /* :181 */
        o.torque_a = v3_cross(r_a, v3_add(slideForceOnA, rollForceA));          /* :184 */
        o.torque_b = v3_cross(r_b, v3_add(v3_neg(slideForceOnA), rollForceA));  /* :185 */
        if (write) {                                                            /* :190-204 */
            const double diffRaRb = s->R[A] - s->R[B];
            const double z = sumRaRb + h;
            const double two_RaRb = 2 * s->R[A] * s->R[B];
            const double denom_sum = z * z - (sumRaRb * sumRaRb);
            const double denom_diff = z * z - (diffRaRb * diffRaRb);
            const double U_vdw = -M->Ha / 6 * (two_RaRb / denom_sum + two_RaRb / denom_diff + log(denom_sum / denom_diff));
            o.pe = U_vdw + 0.5 * k * overlap * overlap;
        }
    } else {
        o.contact = 0;
        double h = fabs(overlap);                                    /* :211-215 */
        if (h < M->h_min) h = M->h_min;
        const double h2 = h * h;
        const double twoRah = 2 * Ra * h;
        const double twoRbh = 2 * Rb * h;
        const double S = h2 + twoRah + twoRbh;
        const double T = h2 + twoRah + twoRbh + 4 * Ra * Rb;
        const double coef = M->Ha / 6 * 64 * Ra * Ra * Ra * Rb * Rb * Rb * ((h + Ra + Rb) / (S * S * T * T));
        o.force_on_a = v3_scale(v3_div(rVecab, v3_norm(rVecab)), coef); /* :221-227 */
        o.torque_a.x = o.torque_a.y = o.torque_a.z = 0;
        o.torque_b = o.torque_a;
        if (write) {                                                 /* :228-240 */
            const double diffRaRb = s->R[A] - s->R[B];
            const double z = sumRaRb + h;
            const double two_RaRb = 2 * s->R[A] * s->R[B];
            const double denom_sum = z * z - (sumRaRb * sumRaRb);
            const double denom_diff = z * z - (diffRaRb * diffRaRb);
            o.pe = -M->Ha / 6 * (two_RaRb / denom_sum + two_RaRb / denom_diff + log(denom_sum / denom_diff));
        }
    }
    return o;
}

static double* dalloc(long n)
{
    double* p = (double*)calloc((size_t)(n > 0 ? n : 1), sizeof(double));
    return p;
}

slo_sys* slo_create(int n, const double* R, const double* m, const double* moi, const slo_material* mat)
{
    if (n < 1) return NULL;
    slo_sys* s = (slo_sys*)calloc(1, sizeof(slo_sys));
    if (!s) return NULL;
    s->n = n;
    s->mat = *mat;
    s->dt = 0; s->kin = 0; s->kout = 0;
    s->pos = dalloc(3L * n); s->vel = dalloc(3L * n); s->velh = dalloc(3L * n);
    s->acc = dalloc(3L * n); s->w = dalloc(3L * n); s->wh = dalloc(3L * n);
    s->aacc = dalloc(3L * n);
    s->R = dalloc(n); s->m = dalloc(n); s->moi = dalloc(n);
    s->distances = dalloc((long)n * (n - 1) / 2);
    s->distances_new = dalloc((long)n * (n - 1) / 2);
    if (!s->pos || !s->vel || !s->velh || !s->acc || !s->w || !s->wh || !s->aacc || !s->R || !s->m ||
        !s->moi || !s->distances || !s->distances_new) {
        slo_destroy(s);
        return NULL;
    }
    memcpy(s->R, R, sizeof(double) * n);
    memcpy(s->m, m, sizeof(double) * n);
    memcpy(s->moi, moi, sizeof(double) * n);
    return s;
}

void slo_destroy(slo_sys* s)
{
    if (!s) return;
    free(s->pos); free(s->vel); free(s->velh); free(s->acc); free(s->w); free(s->wh); free(s->aacc);
    free(s->R); free(s->m); free(s->moi); free(s->distances); free(s->distances_new);
    free(s);
}

int slo_n(const slo_sys* s) { return s->n; }

void slo_set_state(slo_sys* s, const double* pos, const double* vel, const double* w)
{
    memcpy(s->pos, pos, sizeof(double) * 3 * s->n);
    memcpy(s->vel, vel, sizeof(double) * 3 * s->n);
    memcpy(s->w, w, sizeof(double) * 3 * s->n);
}

void slo_set_acc(slo_sys* s, const double* acc, const double* aacc)
{
    memcpy(s->acc, acc, sizeof(double) * 3 * s->n);
    memcpy(s->aacc, aacc, sizeof(double) * 3 * s->n);
}

void slo_set_scalars(slo_sys* s, double dt, double kin, double kout)
{
    s->dt = dt; s->kin = kin; s->kout = kout;
}

void slo_set_prev_positions(slo_sys* s, const double* pos_prev)
{
    for (int A = 1; A < s->n; A++)
        for (int B = 0; B < A; B++)
            s->distances[tri_index(A, B)] = v3_norm(v3_sub(v3_at(pos_prev, B), v3_at(pos_prev, A)));
}

/* Pass 1, ColliderSingleCore.cpp:82-97. */
static void pass1(slo_sys* s)
{
    const double dt = s->dt;
    for (long b = 0; b < s->n; b++) {
        const v3 velh = v3_add(v3_at(s->vel, b), v3_scale(v3_scale(v3_at(s->acc, b), .5), dt));
        const v3 wh = v3_add(v3_at(s->w, b), v3_scale(v3_scale(v3_at(s->aacc, b), .5), dt));
        const v3 pos = v3_add(v3_at(s->pos, b), v3_scale(velh, dt));
        s->velh[3 * b] = velh.x; s->velh[3 * b + 1] = velh.y; s->velh[3 * b + 2] = velh.z;
        s->wh[3 * b] = wh.x; s->wh[3 * b + 1] = wh.y; s->wh[3 * b + 2] = wh.z;
        s->pos[3 * b] = pos.x; s->pos[3 * b + 1] = pos.y; s->pos[3 * b + 2] = pos.z;
        s->acc[3 * b] = s->acc[3 * b + 1] = s->acc[3 * b + 2] = 0;
        s->aacc[3 * b] = s->aacc[3 * b + 1] = s->aacc[3 * b + 2] = 0;
    }
}

static inline void add_to(double* a, long i, v3 v) { a[3 * i] += v.x; a[3 * i + 1] += v.y; a[3 * i + 2] += v.z; }
static inline void sub_from(double* a, long i, v3 v) { a[3 * i] -= v.x; a[3 * i + 1] -= v.y; a[3 * i + 2] -= v.z; }

/* Pass 2 in the reference's loop order, ColliderSingleCore.cpp:100-256. */
static double pass2_seq(slo_sys* s, int write)
{
    double PE = 0;
    for (int A = 1; A < s->n; A++) {
        for (int B = 0; B < A; B++) {
            const long e = tri_index(A, B);
            const pair_out o = pair_eval(s, A, B, s->distances[e], write);
            if (o.contact) {
                add_to(s->aacc, A, v3_div(o.torque_a, s->moi[A])); /* :187 */
                add_to(s->aacc, B, v3_div(o.torque_b, s->moi[B])); /* :188 */
            }
            if (write) PE += o.pe;
            add_to(s->acc, A, v3_div(o.force_on_a, s->m[A]));       /* :249 */
            sub_from(s->acc, B, v3_div(o.force_on_a, s->m[B]));     /* :250 */
            s->distances[e] = o.dist;                               /* :253 */
        }
    }
    return PE;
}

/* Pass 2 row-parallel: sphere i receives its terms in ascending partner
 * order (partners j<i while i is A, then j>i while i is B), which is the
 * order in which the reference loop adds them to acc[i] and aacc[i]. */
static double pass2_rows(slo_sys* s, int write, int nthreads)
{
    const int n = s->n;
    double PE = 0;
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 8) num_threads(nthreads) reduction(+ : PE)
#endif
    for (int i = 0; i < n; i++) {
        v3 acc = {0, 0, 0}, aacc = {0, 0, 0};
        double pe_row = 0;
        for (int j = 0; j < n; j++) {
            if (j == i) continue;
            const int A = i > j ? i : j, B = i > j ? j : i;
            const long e = tri_index(A, B);
            const pair_out o = pair_eval(s, A, B, s->distances[e], write);
            if (i == A) {
                if (o.contact) aacc = v3_add(aacc, v3_div(o.torque_a, s->moi[A]));
                acc = v3_add(acc, v3_div(o.force_on_a, s->m[A]));
                s->distances_new[e] = o.dist;
                if (write) pe_row += o.pe;
            } else {
                if (o.contact) aacc = v3_add(aacc, v3_div(o.torque_b, s->moi[B]));
                acc = v3_sub(acc, v3_div(o.force_on_a, s->m[B]));
            }
        }
        s->acc[3 * i] = acc.x; s->acc[3 * i + 1] = acc.y; s->acc[3 * i + 2] = acc.z;
        s->aacc[3 * i] = aacc.x; s->aacc[3 * i + 1] = aacc.y; s->aacc[3 * i + 2] = aacc.z;
        PE += pe_row;
    }
    double* t = s->distances; s->distances = s->distances_new; s->distances_new = t;
    return PE;
}

/* Pass 3, ColliderSingleCore.cpp:263-287. */
static void pass3(slo_sys* s, int write, double PE, double* e)
{
    const double dt = s->dt;
    double KE = 0;
    v3 mom = {0, 0, 0}, L = {0, 0, 0};
    for (long b = 0; b < s->n; b++) {
        const v3 vel = v3_add(v3_at(s->velh, b), v3_scale(v3_scale(v3_at(s->acc, b), .5), dt));
        const v3 w = v3_add(v3_at(s->wh, b), v3_scale(v3_scale(v3_at(s->aacc, b), .5), dt));
        s->vel[3 * b] = vel.x; s->vel[3 * b + 1] = vel.y; s->vel[3 * b + 2] = vel.z;
        s->w[3 * b] = w.x; s->w[3 * b + 1] = w.y; s->w[3 * b + 2] = w.z;
        if (write) {
            KE += .5 * s->m[b] * v3_norm2(vel) + .5 * s->moi[b] * v3_norm2(w);          /* :282-283 */
            mom = v3_add(mom, v3_scale(vel, s->m[b]));                                   /* :284 */
            L = v3_add(L, v3_add(v3_scale(v3_cross(v3_at(s->pos, b), vel), s->m[b]),     /* :285 */
                                 v3_scale(w, s->moi[b])));
        }
    }
    if (write && e) {
        e[SLO_E_PE] = PE; e[SLO_E_KE] = KE;
        e[SLO_E_MOM] = mom.x; e[SLO_E_MOM + 1] = mom.y; e[SLO_E_MOM + 2] = mom.z;
        e[SLO_E_L] = L.x; e[SLO_E_L + 1] = L.y; e[SLO_E_L + 2] = L.z;
    }
}

void slo_init(slo_sys* s, double* energy_out)
{
    /* distances := current distances (the reference reads an uninitialised
     * array here, ball_group.hpp:741,796; current distances make the initial
     * contacts take k = kout, which the GPU path reproduces). */
    slo_set_prev_positions(s, s->pos);
    const double dt = s->dt;
    s->dt = 0; /* with dt = 0 passes 1 and 3 leave pos/vel/w unchanged */
    pass1(s);
    const double PE = pass2_seq(s, 1);
    pass3(s, 1, PE, energy_out);
    s->dt = dt;
}

void slo_step(slo_sys* s, int write, double* energy_out)
{
    pass1(s);
    const double PE = pass2_seq(s, write);
    pass3(s, write, PE, energy_out);
}

void slo_step_rows(slo_sys* s, int write, double* energy_out, int nthreads)
{
    pass1(s);
    const double PE = pass2_rows(s, write, nthreads);
    pass3(s, write, PE, energy_out);
}

void slo_get_state(const slo_sys* s, double* pos, double* vel, double* w, double* acc, double* aacc)
{
    const size_t bytes = sizeof(double) * 3 * s->n;
    if (pos) memcpy(pos, s->pos, bytes);
    if (vel) memcpy(vel, s->vel, bytes);
    if (w) memcpy(w, s->w, bytes);
    if (acc) memcpy(acc, s->acc, bytes);
    if (aacc) memcpy(aacc, s->aacc, bytes);
}

long slo_contacts(const slo_sys* s, int* pairs, long max_pairs)
{
    long count = 0;
    for (int A = 1; A < s->n; A++)
        for (int B = 0; B < A; B++) {
            const double dist = v3_norm(v3_sub(v3_at(s->pos, B), v3_at(s->pos, A)));
            if (s->R[A] + s->R[B] - dist > 0) {
                if (pairs && count < max_pairs) { pairs[2 * count] = A; pairs[2 * count + 1] = B; }
                count++;
            }
        }
    return count;
}

int slo_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
