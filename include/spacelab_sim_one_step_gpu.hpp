/*
 * spacelab_sim_one_step_gpu.hpp -- the reference-side adapter: SpaceLab's
 * sim_one_step (ColliderSingleCore/ColliderSingleCore.cpp:78-288) run on the
 * GPU through the C ABI of spacelab_gpu.h.
 *
 * This header is meant to be included INTO ColliderSingleCore.cpp, after the
 * global `Ball_group O` (ColliderSingleCore.cpp:33), because it works on the
 * reference's own globals: O, dt, kin, kout (dust_const.hpp:51-53), the
 * material constants G, Ha, u_s, u_r, h_min (dust_const.hpp:21-38) and the
 * simData row buffer `ballBuffer` (ColliderSingleCore.cpp:12).  A
 * maintainer's edit of ColliderSingleCore.cpp is:
 *
 *   1. `#include "spacelab_sim_one_step_gpu.hpp"` after line 33;
 *   2. in sim_looper, `sim_one_step_gpu(writeStep);` instead of
 *      `sim_one_step(writeStep);` (line 331);
 *   3. `sl_gpu_begin();` once O is set up and dt/kin/kout are set (after
 *      `O.sim_init_write(...)` in main, before `sim_looper()`), and
 *      `sl_gpu_sync_host();` before anything else reads O's arrays.
 *
 * Build: -I<this repo>/include, link libspacelab_gb300.so.
 *
 * What sim_one_step_gpu does on a write step, as the reference's pass 2/3 do:
 * adds the step's PE, KE, momentum and angular momentum into O.PE, O.KE,
 * O.mom, O.ang_mom (ColliderSingleCore.cpp:190-204, 228-240, 282-285), copies
 * the state back into O and appends the pass-3 row of simData.csv to
 * ballBuffer (:257-281): per sphere x, y, z, wx, wy, wz, |w|, vx, vy, vz and
 * the bound flag 0, so sim_looper's file export (:350-360) writes the same
 * files as with the CPU step.  Errors print sl_last_error() and exit, the
 * reference's own error style.
 */
#ifndef SPACELAB_SIM_ONE_STEP_GPU_HPP
#define SPACELAB_SIM_ONE_STEP_GPU_HPP

#include "spacelab_gpu.h"

#include <cstdio>
#include <cstdlib>

// The one GPU system the reference's single global O maps to.
inline sl_handle*& sl_gpu_handle()
{
    static sl_handle* h = nullptr;
    return h;
}

inline void sl_gpu_check(int rc, const char* where)
{
    if (rc != SL_OK) {
        fprintf(stderr, "%s: %s\n", where, sl_last_error());
        exit(EXIT_FAILURE);
    }
}

// Free the GPU copy of O (safe to call when there is none).
inline void sl_gpu_end()
{
    sl_destroy(sl_gpu_handle());
    sl_gpu_handle() = nullptr;
}

// Copy O to the GPU and compute its initial forces there (init_conditions,
// ball_group.hpp:777-947).  Call again whenever O is replaced (the
// reference's main rebuilds O with add_projectile before each sim_looper).
inline void sl_gpu_begin()
{
    sl_gpu_end();
    const sl_material mat{G, Ha, u_s, u_r, h_min};
    sl_handle*& h = sl_gpu_handle();
    sl_gpu_check(sl_create(O.num_particles, &mat, SL_MODE_EXACT, &h), "sl_create");
    // vec3 is three contiguous doubles (vec3.hpp:10-15), so &v[0].x is a double[3n]
    sl_gpu_check(sl_upload(h, &O.pos[0].x, &O.vel[0].x, &O.w[0].x, O.R, O.m, O.moi), "sl_upload");
    sl_gpu_check(sl_set_scalars(h, dt, kin, kout), "sl_set_scalars");
    sl_gpu_check(sl_init_forces(h, nullptr), "sl_init_forces");
}

// Copy the GPU state back into O's arrays.
inline void sl_gpu_sync_host()
{
    sl_gpu_check(sl_download(sl_gpu_handle(), &O.pos[0].x, &O.vel[0].x, &O.w[0].x, &O.acc[0].x, &O.aacc[0].x),
                 "sl_download");
}

// Drop-in for sim_one_step(write_step).  If dt/kin/kout change between
// steps (dynamicTime, ColliderSingleCore.cpp:373), call
// sl_set_scalars(sl_gpu_handle(), dt, kin, kout) after the change.
inline void sim_one_step_gpu(const bool write_step)
{
    sl_energy e;
    sl_gpu_check(sl_step(sl_gpu_handle(), 1, write_step ? 1 : 0, &e), "sl_step");
    if (!write_step) return;
    O.PE += e.PE;
    O.KE += e.KE;
    O.mom += vec3(e.mom[0], e.mom[1], e.mom[2]);
    O.ang_mom += vec3(e.ang_mom[0], e.ang_mom[1], e.ang_mom[2]);
    sl_gpu_sync_host();
    // the simData.csv row of this write step, in the reference's column order
    ballBuffer << '\n';
    for (int i = 0; i < O.num_particles; i++) {
        if (i > 0) ballBuffer << ',';
        const vec3& p = O.pos[i];
        const vec3& w = O.w[i];
        const vec3& v = O.vel[i];
        ballBuffer << p.x << ',' << p.y << ',' << p.z << ',' << w.x << ',' << w.y << ',' << w.z << ','
                   << w.norm() << ',' << v.x << ',' << v.y << ',' << v.z << ',' << 0;
    }
}

#endif /* SPACELAB_SIM_ONE_STEP_GPU_HPP */
