// sl_batch.h -- device layout of a batch of independent systems (one
// projectile-target collision each) advanced by one persistent launch.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "sl_device.cuh"

namespace sl {

// Energy record layout: [inst][rec][8] = PE, KE, mom xyz, ang_mom xyz.
struct Batch {
    int ninst;
    int total;            // spheres over all instances
    const int* order;     // instance processing order (largest first)
    int* counter;         // work-queue head
    const int* off;       // first sphere of each instance
    const int* cnt;       // spheres of each instance
    const double* dt;     // per-instance time step
    const double* kin;    // per-instance spring constants
    const double* kout;
    const double* u_s;    // per-instance sliding friction
    Vec3Soa pos, prev, vel, velh, w, wh, acc, aacc;
    double *R, *m, *moi, *twoR, *fourR, *cR3;
    unsigned long long* rm;  // 64-bit fixed-point reciprocal significand of m (recip_sig)
    double* inv_moi;
    // Mixed form.  Its pair passes see each instance's spheres in "slots":
    // perm[off + k] = off + the instance's k-th sphere in Z-order of its
    // positions at upload, so that a warp's spheres, and a 32-slot block, are
    // close together and few of them take the close-pair path.  The FP32
    // arrays below are in slot order (entry off + k belongs to sphere
    // perm[off + k]); the FP64 state stays in the caller's order.
    const int* perm;
    float *f_R, *f_inv_m, *f_inv_moi;  // lengths scaled by 2^-len_shift
    // the radii's double-float lo parts, and the positions as double-float
    // hi (x, y, z) and lo (x, y, z), written by the drift
    float *f_Rlo, *f_pos[6];
    float far_sq;  // far-pair threshold (far_threshold_sq in sl_pair_mixed.cuh)
    // mixed form, pair-tile pass (shape tile 0): per-CTA scratch of tile
    // partials, CTA c at part + c * part_cta, [6][part_nb][part_np] floats
    float* part;
    size_t part_cta;
    int part_nb, part_np, part_ctas;  // part_ctas: CTAs the pair-tile scratch exists for (either form)
    // exact form, pair-tile pass (shape tile 0): per-CTA pair-term and torque
    // buffers [3][x_np][x_np] doubles and contact words [x_np][x_nb], the
    // single-system layout at a fixed stride; NULL where the largest
    // instance makes them too big
    double *xpair, *xtorq;
    uint32_t* xmask;
    size_t xpair_cta, xmask_cta;
    int x_np, x_nb;
    Scalars* isc;  // per-instance dt, kin, kout as one record (the exact tile pass's System view)
    int len_shift;
    Material mat;         // G, Ha, u_r, h_min shared; u_s per instance
    double* energy;       // [ninst][nrec][8]
    int nrec;
    unsigned* status;     // per instance: 1 = non-finite state
};

// CTAs per SM the pair-tile pass's scratch is sized for.
constexpr int kTileCtasPerSm = 4;

// Launch the persistent kernel over all instances: an initial force pass
// when do_init, then steps first_step .. first_step+nsteps-1 with a write
// (energy record) at every step divisible by skip.  Records: rec 0 = the
// initial pass, rec k = after step k*skip.
void launch_batch_exact(const Batch& b, int tile, int threads, int blocks, int first_step, int nsteps, int skip,
                        int do_init, cudaStream_t st);
void launch_batch_mixed(const Batch& b, int tile, int threads, int blocks, int first_step, int nsteps, int skip,
                        int do_init, cudaStream_t st);
void launch_batch_derive(const Batch& b, cudaStream_t st);
int batch_max_blocks_per_sm(int tile, int threads, bool mixed);
int batch_mixed_max_blocks_per_sm(int tile, int threads);

}  // namespace sl
