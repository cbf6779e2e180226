/*
 * spacelab_batch.h -- C ABI of the batched solver (libspacelab_gb300.so):
 * thousands of independent systems -- one projectile-target collision each,
 * of uneven sphere counts -- advanced by ONE persistent, graph-captured
 * launch.  No counterpart in the reference, which runs one system per
 * process (its add_projectile loop, ColliderSingleCore.cpp:64-71, is
 * serial); each instance's step is the reference's sim_one_step
 * (ColliderSingleCore.cpp:78-288), and in SL_MODE_EXACT an instance's state
 * is bit-identical to running it alone through sl_step.
 *
 * Layout: instance i owns spheres [off_i, off_i + counts[i]) of the
 * concatenated arrays (off_i = counts[0] + ... + counts[i-1]); pos/vel/w/
 * acc/aacc are vec3[total] (3 doubles per sphere), R/m/moi double[total].
 * Per-instance parameters: dt, kin, kout (restitution) and u_s (sliding
 * friction); G, Ha, u_r and h_min are shared (sl_material; its u_s is
 * unused).  Energy records per instance: rec 0 from the initial force pass,
 * rec k after step k*skip, 8 doubles each (PE, KE, mom xyz, ang_mom xyz).
 */
#ifndef SPACELAB_BATCH_H
#define SPACELAB_BATCH_H

#include "spacelab_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct sl_batch sl_batch;

/* Allocate a batch for `steps` steps with an energy record every `skip`. */
int sl_batch_create(int ninst, const int* counts, const sl_material* mat, int mode, int steps, int skip,
                    sl_batch** out);
int sl_batch_destroy(sl_batch* b);

/* Copy the concatenated state and the per-instance parameters (host arrays). */
int sl_batch_upload(sl_batch* b, const double* pos, const double* vel, const double* w, const double* R,
                    const double* m, const double* moi, const double* dt, const double* kin, const double* kout,
                    const double* u_s);

/* Launch shape: j-tile size (32, 64, 128 spheres staged in shared memory)
 * and threads per instance (64, 128, 256 = the block size).  Tile 0
 * selects the pair-tile pass instead, every pair evaluated once in 32 x 32
 * blocks: in the mixed form over Z-ordered spheres with per-CTA partial sums
 * (also at 512 threads); in the exact form with per-CTA pair-term buffers and
 * ordered row sums, bit-identical to the other shapes (SL_ERR_UNSUPPORTED
 * where the largest instance makes those buffers too big). */
int sl_batch_set_shape(sl_batch* b, int tile, int threads);
int sl_batch_shape(const sl_batch* b, int* tile, int* threads, int* blocks);

/* Autotuner: times every tile x threads candidate on sample_steps steps of
 * the whole batch (from a saved copy of the current state, restored
 * afterwards), keeps the fastest and returns it; times_ms (12 entries,
 * tile-major in the order 32, 64, 128, 0, threads 64, 128, 256 -- for tile
 * 0 in the mixed form: 128, 256, 512 -- may be NULL) gets each candidate's
 * time, -1 where tile 0 is unavailable. */
int sl_batch_autotune(sl_batch* b, int sample_steps, int* tile, int* threads, double* times_ms);

/* One persistent launch: the initial force pass if do_init, then steps
 * first_step .. first_step+nsteps-1 of every instance. */
int sl_batch_run(sl_batch* b, int first_step, int nsteps, int do_init);

int sl_batch_download(sl_batch* b, double* pos, double* vel, double* w, double* acc, double* aacc);
/* energy: [ninst][nrec][8]; *nrec = steps / skip + 1. */
int sl_batch_energy(sl_batch* b, double* energy, int* nrec);
/* Per instance: 0, or 1 when its state became non-finite. */
int sl_batch_status(sl_batch* b, unsigned* status);

#ifdef __cplusplus
}
#endif
#endif /* SPACELAB_BATCH_H */
