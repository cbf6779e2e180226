/*
 * spacelab_gpu.h -- C ABI of the GB300 step library (libspacelab_gb300.so).
 *
 * Drop-in for the per-step hot path of SpaceLab: the reference's
 * `void sim_one_step(const bool write_step)` (ColliderSingleCore/
 * ColliderSingleCore.cpp:24-25,78-288) operating on the global
 * `Ball_group O` (ball_group.hpp:18-53) and the mutable globals
 * dt/kin/kout (dust_const.hpp:51-53).  The reference has no FFI of its own:
 * its "interface" is those globals plus raw `vec3*` arrays, so every entry
 * point below takes plain pointers to the same memory a Ball_group holds:
 * `pos`, `vel`, `w`, `acc`, `aacc` are arrays of 3n doubles laid out as the
 * reference's `vec3[n]` (x, y, z per sphere; vec3.hpp:10-15), and R, m, moi
 * are arrays of n doubles.
 *
 * Conventions
 *   - Every function returns an int status (SL_OK == 0).  Nothing calls
 *     exit(): the reference's exit(EXIT_FAILURE) paths (ColliderSingleCore.cpp
 *     :387-444) become SL_ERR_ARG / SL_ERR_NONFINITE returns, and
 *     sl_last_error() gives a one-line reason.
 *   - A handle owns device copies of one system's arrays; host arrays stay
 *     owned by the caller.  Calls on one handle are serialised on the
 *     handle's CUDA stream and are not thread-safe; use one handle per host
 *     thread.  Handles are independent of each other.
 *   - Results of SL_MODE_EXACT are bit-identical to the reference's step
 *     compiled with IEEE double arithmetic and no contraction (MSVC
 *     /fp:precise, g++ -ffp-contract=off); energy totals are summed in a
 *     different order and agree to rounding.
 */
#ifndef SPACELAB_GPU_H
#define SPACELAB_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SL_API_VERSION 2

/* status codes */
#define SL_OK 0
#define SL_ERR_ARG 1        /* bad argument (n < 1, NULL, non-positive R/m/moi, ...) */
#define SL_ERR_CUDA 2       /* CUDA runtime error (no device, launch failure) */
#define SL_ERR_NONFINITE 3  /* a position/velocity/spin became NaN or Inf */
#define SL_ERR_ALLOC 4      /* device or host allocation failed */
#define SL_ERR_STATE 5      /* call out of order (e.g. step before upload) */
#define SL_ERR_UNSUPPORTED 6
#define SL_ERR_TIMEOUT 7     /* a kernel's bounded wait for its own asynchronous copies ran out */

/* arithmetic modes of the pair step */
#define SL_MODE_EXACT 0     /* FP64, reference operation order, bit-exact */
#define SL_MODE_MIXED 1     /* FP32 force and torque arithmetic on relative
                               displacements; FP64 positions, pair subtraction
                               r_i - r_j, overlaps of close pairs, per-sphere
                               force/torque accumulation and energy sums;
                               deterministic, not bit-exact */
#define SL_MODE_MIXED_DF 2  /* no FP64 pipe work for pairs out of contact:
                               double-float (FP32 hi + lo, ~48 bits) pair
                               subtraction and overlap of close pairs, FP32
                               per-tile partial sums added in compensated
                               double-float; FP64 positions, integration,
                               contact k choice and energy totals;
                               deterministic, not bit-exact */

/* Material constants that the reference compiles in (dust_const.hpp:21-38):
 * G, Hamaker constant Ha, sliding and rolling friction u_s and u_r, and the
 * minimum vdW separation h_min.  Units are cgs. */
typedef struct sl_material {
    double G;
    double Ha;
    double u_s;
    double u_r;
    double h_min;
} sl_material;

/* Totals of one write step, as accumulated into Ball_group's PE, KE, mom and
 * ang_mom by sim_one_step (ColliderSingleCore.cpp:190-204, 228-240, 282-285). */
typedef struct sl_energy {
    double PE;
    double KE;
    double mom[3];
    double ang_mom[3];
} sl_energy;

typedef struct sl_handle sl_handle;

/* Library version (SL_API_VERSION) -- lets a loader check the ABI. */
int sl_version(void);

/* One-line description of the last error on this host thread. */
const char* sl_last_error(void);

/* Allocate a system of n spheres on the current CUDA device.
 * Replaces Ball_group::allocate_group (ball_group.hpp:736-756) plus the
 * compiled-in constants of dust_const.hpp:21-38.
 * 1 <= n <= 46340: beyond that the reference's own pair index
 * A(A-1)/2+B of its `distances` array overflows an int (ball_group.hpp:741),
 * so the reference cannot run such a system to compare with.  The GPU keeps
 * no such array; the limit is kept so that every system accepted here is
 * one the reference can run.  Device memory grows as 48 npad^2 bytes in
 * SL_MODE_EXACT (pair and torque terms; 103 GB at the limit), and a failed
 * allocation returns SL_ERR_ALLOC. */
int sl_create(int n, const sl_material* mat, int mode, sl_handle** out);

/* Free everything the handle owns.  Replaces Ball_group::freeMemory
 * (ball_group.hpp:760-773).  NULL is accepted. */
int sl_destroy(sl_handle* h);

/* Number of spheres (Ball_group::num_particles, ball_group.hpp:21). */
int sl_num_particles(const sl_handle* h, int* n);

/* Copy a Ball_group's state to the device: pos/vel/w as vec3[n], R/m/moi as
 * double[n] (ball_group.hpp:44-53).  acc/aacc are zeroed; previous-step
 * distances are set to the current ones.  R, m, moi must be > 0. */
int sl_upload(sl_handle* h, const double* pos, const double* vel, const double* w, const double* R,
              const double* m, const double* moi);

/* Resume an exact state: also sets acc/aacc (vec3[n]) and the positions of
 * the previous step (vec3[n]; the reference's `distances`, ball_group.hpp:741,
 * are the pair distances of those positions).  NULL pos_prev = pos. */
int sl_upload_resume(sl_handle* h, const double* pos, const double* vel, const double* w,
                     const double* acc, const double* aacc, const double* pos_prev);

/* Set the mutable step scalars dt, kin, kout (dust_const.hpp:51-53;
 * ball_group.hpp:1313-1329 computes them in the reference). */
int sl_set_scalars(sl_handle* h, double dt, double kin, double kout);

/* Initial force pass (Ball_group::init_conditions, ball_group.hpp:777-947):
 * acc/aacc and, in *out (may be NULL), the initial PE/KE/mom/ang_mom.
 * Initially touching pairs take k = kout (their previous distance equals
 * the current one). */
int sl_init_forces(sl_handle* h, sl_energy* out);

/* Run nsteps reference steps (sim_one_step, ColliderSingleCore.cpp:78-288).
 * Only the last step is a write step, and only if write_last != 0; its
 * totals go to *out (may be NULL).  Returns SL_ERR_NONFINITE if the state
 * became non-finite (checked at write steps and at the end). */
int sl_step(sl_handle* h, int nsteps, int write_last, sl_energy* out);

/* The loop of sim_looper (ColliderSingleCore.cpp:291-375): steps
 * first_step .. last_step-1, a write step whenever step % skip == 0, one
 * energy row per write step into rows[0..max_rows).  *nrows gets the number
 * of rows written.  The steps between writes run as one CUDA graph. */
int sl_run(sl_handle* h, int first_step, int last_step, int skip, sl_energy* rows, int max_rows,
           int* nrows);

/* Copy the device state back into Ball_group-shaped arrays (any may be
 * NULL): pos, vel, w, acc, aacc as vec3[n]. */
int sl_download(sl_handle* h, double* pos, double* vel, double* w, double* acc, double* aacc);

/* One reference step on a state the caller keeps on the host: the drop-in
 * for sim_one_step(write) (ColliderSingleCore.cpp:78-288) when the host owns
 * O.pos/vel/w/acc/aacc and may change them between steps.  Reads the five
 * vec3[n] arrays (the end of the caller's previous step; its previous-step
 * positions are taken as pos, as the reference's `distances` hold the
 * current positions' pair distances between steps), runs the step, and
 * writes the new state back into the same arrays; a write step's totals go
 * to *out (may be NULL).  The same bits as sl_upload_resume(h, pos, vel, w,
 * acc, aacc, NULL) + sl_step(h, 1, write, out) + sl_download(h, pos, vel,
 * w, acc, aacc), with one wait for the GPU instead of three.  Requires
 * sl_upload (R, m, moi) first; pos, vel, w, acc, aacc non-NULL.  A NaN or
 * Inf in pos, vel or w returns SL_ERR_ARG and leaves the five arrays as they
 * were (*out is then undefined); the handle's device copy of the state is
 * undefined until the next successful upload or sl_step_host. */
int sl_step_host(sl_handle* h, double* pos, double* vel, double* w, double* acc, double* aacc, int write,
                 sl_energy* out);

/* Contact pairs (A > B, overlap R[A]+R[B]-|pos[B]-pos[A]| > 0) found by the
 * last force pass, in the reference's loop order (A ascending, then B
 * ascending; ColliderSingleCore.cpp:100-119).  Writes min(count, max_pairs)
 * (A, B) int pairs; *count gets the total. */
int sl_contacts(sl_handle* h, int* pairs, long max_pairs, long* count);

/* The handle's CUDA stream (a cudaStream_t), for callers that order their
 * own work or timing events against the library's launches. */
void* sl_stream(sl_handle* h);

/* Exact mode can pipeline each step: the pair tiles run in five
 * block-column phases on the handle's stream, and the row sums over each
 * phase's partner blocks run on a second stream while the later phases
 * compute.  The sums keep their order, so results are bit-identical either
 * way.  Both kernels are limited by the FP64 pipe, so the overlap pays only
 * where the row sums are latency-bound and the phases stay large (about
 * +0.7% at N=20000, -5% at N=5000 on GB300).  Default: disabled.  The
 * mixed modes have no pipelined form (SL_ERR_UNSUPPORTED for enable != 0). */
int sl_set_overlap(sl_handle* h, int enable);

/* How exact mode adds each sphere's pair terms in the reference's order
 * (ColliderSingleCore.cpp:249-250).  SL_ROWSUM_FP64 (the default) uses
 * the FP64 unit; SL_ROWSUM_INT computes every FP64 addition, correctly
 * rounded, on the integer pipe.  The sums are identical bit for bit either
 * way; only the time differs.  Exact mode only (SL_ERR_UNSUPPORTED for the
 * mixed modes, which keep no per-pair terms). */
#define SL_ROWSUM_INT 0
#define SL_ROWSUM_FP64 1
int sl_set_rowsum(sl_handle* h, int method);

/* Kernel launches one step makes (a write step computes the energy too). */
int sl_step_launches(const sl_handle* h, int write, int* count);

/* Name of the pair kernel the handle's steps launch: "pair_tile_kernel"
 * (exact mode), "mixed64_pair_kernel" (SL_MODE_MIXED), "mixed_pair_kernel"
 * or, for large systems, "mixed_pair2_kernel" (two column blocks per work
 * item; SL_MODE_MIXED_DF).  The string is static. */
int sl_pair_kernel(const sl_handle* h, const char** name);

/* Per-kernel timing: when enabled, every step records CUDA events around
 * the pair kernel and the row-sum kernel; sl_kernel_times returns their
 * accumulated milliseconds and launch counts since the last reset.  With
 * the pipelined step, "pair" spans all pair phases (the row sums of the
 * earlier phases run inside it) and "row-sum" is the part of the row sums
 * left after the last pair phase. */
int sl_kernel_timing(sl_handle* h, int enable);
int sl_kernel_times(sl_handle* h, double* pair_ms, double* rowsum_ms, long* launches, int reset);

/* Bytes of device memory the handle holds. */
int sl_device_bytes(const sl_handle* h, uint64_t* bytes);

/* Largest system sl_forces_static accepts. */
#define SL_STATIC_MAX_SPHERES 256

/* The initial force pass (what sl_init_forces computes) for a system that
 * lives in the caller's own device memory, without allocating anything.
 * No counterpart in the reference: it exists for callers that cannot call
 * cudaMalloc -- code running inside a host application that owns and
 * budgets all device memory and hands its plugins ready-made buffers, and
 * code on a real-time path where an allocation's implicit device
 * synchronisation and unbounded latency are not allowed.
 *
 * All pointers except mat are DEVICE pointers owned by the caller:
 *   pos, vel, w      vec3[n] inputs (3n doubles each, x y z per sphere)
 *   R, m, moi        double[n] inputs, each > 0
 *   acc, aacc        vec3[n] outputs
 *   energy           8 doubles out (PE, KE, mom xyz, ang_mom xyz), or NULL
 * stream is a cudaStream_t (NULL = the legacy default stream); the call
 * returns after the work on it has finished.  Initially touching pairs take
 * k = kout, as in sl_init_forces.
 *
 * Limit: 1 <= n <= SL_STATIC_MAX_SPHERES; larger n returns SL_ERR_ARG, and
 * so does a sphere whose R, m or moi is not finite and > 0.
 * Working memory is one static device array of about 3.2 MB that every GPU
 * loading this library holds until the process exits.  The first call on a
 * device looks up that array's device address (cudaGetSymbolAddress), so make
 * the first call on each device before any stream capture.  The address is
 * looked up again when the current context is another one than the one it
 * came from (after cudaDeviceReset, or under a driver-API context of the
 * caller's own), so calls after a reset work.  All calls share the array:
 * calls whose work overlaps on the GPU (other host threads, or other
 * streams) race and must be serialised by the caller. */
int sl_forces_static(int n, const double* pos, const double* vel, const double* w, const double* R,
                     const double* m, const double* moi, const sl_material* mat, double kin, double kout,
                     double* acc, double* aacc, double* energy, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* SPACELAB_GPU_H */
