/*
 * sl_oracle.h -- CPU oracle for the SpaceLab step (TEST INFRASTRUCTURE ONLY).
 *
 * This is a plain-C restatement of the reference's per-step hot path, used
 * only as the checker by the test suite, by smoke() and by the CPU-baseline
 * legs of bench.py.  It is never linked into, loaded by or called from the
 * GPU product library.
 *
 * Reference being restated (paths inside the SpaceLab project):
 *   ColliderSingleCore/ColliderSingleCore.cpp:78-288   sim_one_step (3 passes)
 *   ball_group.hpp:777-947                             init_conditions
 *   vec3.hpp:44-128,180-184                            vec3 operation order
 *   ball_group.hpp:42-53, 736-756                      Ball_group arrays
 *
 * The restatement keeps the reference's O(N^2) `distances` array (previous
 * step pair distances, triangular index A*(A-1)/2+B) so that it is a literal
 * restatement; the GPU path replaces it with previous positions.
 *
 * Parity pin: slo_step() is checked bit-for-bit against the reference's own
 * sim_one_step compiled from the unmodified reference sources (oracle/_ref,
 * built by oracle/Makefile in a container that has the reference) by
 * tests/test_oracle_pin.py, and against committed golden vectors generated by
 * that build (tests/golden/make_golden.py).
 */
#ifndef SL_ORACLE_H
#define SL_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

typedef struct slo_material {
    double G;      /* gravitational constant            dust_const.hpp:21 */
    double Ha;     /* Hamaker constant                  dust_const.hpp:37 */
    double u_s;    /* sliding friction coefficient      dust_const.hpp:23 */
    double u_r;    /* rolling friction coefficient      dust_const.hpp:24 */
    double h_min;  /* minimum vdW separation            dust_const.hpp:38 */
} slo_material;

typedef struct slo_sys slo_sys;

/* Energy record of one write step: PE, KE, mom[3], ang_mom[3]. */
enum { SLO_E_PE = 0, SLO_E_KE = 1, SLO_E_MOM = 2, SLO_E_L = 5, SLO_E_COUNT = 8 };

slo_sys* slo_create(int n, const double* R, const double* m, const double* moi,
                    const slo_material* mat);
void slo_destroy(slo_sys* s);
int slo_n(const slo_sys* s);
void slo_set_state(slo_sys* s, const double* pos, const double* vel, const double* w);
void slo_set_acc(slo_sys* s, const double* acc, const double* aacc);
void slo_set_scalars(slo_sys* s, double dt, double kin, double kout);
/* Overwrite the previous-step pair distances with the distances of `pos_prev`
 * (AoS xyz).  Used to resume from a saved state. */
void slo_set_prev_positions(slo_sys* s, const double* pos_prev);

/* Initial force pass (ball_group.hpp:777-947): distances := current pair
 * distances, then one pass-2 evaluation with write=1; acc/aacc start at 0.
 * energy_out (8 doubles, may be NULL) gets PE and KE/mom/ang_mom. */
void slo_init(slo_sys* s, double* energy_out);

/* One reference step (ColliderSingleCore.cpp:78-288), sequential loops in
 * the reference order.  energy_out is filled when write != 0. */
void slo_step(slo_sys* s, int write, double* energy_out);

/* Same step computed row-parallel (each sphere sums its pair terms in
 * ascending partner order, which is the reference's accumulation order), on
 * `nthreads` OpenMP threads (0 = all).  pos/vel/w/acc/aacc are bit-identical
 * to slo_step; the PE/KE/mom/L totals are summed in another order. */
void slo_step_rows(slo_sys* s, int write, double* energy_out, int nthreads);

void slo_get_state(const slo_sys* s, double* pos, double* vel, double* w,
                   double* acc, double* aacc);

/* Pairs (A > B) with overlap R[A]+R[B]-|pos[B]-pos[A]| > 0 at the current
 * positions, in reference loop order; returns the count (writes at most
 * max_pairs pairs as A,B int pairs). */
long slo_contacts(const slo_sys* s, int* pairs, long max_pairs);

/* Step count of slo_step_rows runs on this many threads when nthreads==0. */
int slo_max_threads(void);

#ifdef __cplusplus
}
#endif
#endif
