// ref_harness.cpp -- builds the reference's own sim_one_step as a shared
// library for pinning the oracle (TEST INFRASTRUCTURE ONLY).
//
// Compiles the UNMODIFIED reference translation unit
// ColliderSingleCore/ColliderSingleCore.cpp (which includes ball_group.hpp,
// dust_const.hpp, vec3.hpp, Utils.hpp, linalg.hpp) from the reference tree
// given by -I<reference root>; nothing of the reference is copied here.
// Adaptations, all outside the reference's code:
//   * `using std::isnan;` so the unqualified isnan at ball_group.hpp:1419
//     resolves under g++ 13;
//   * the material constants of dust_const.hpp:21-38 are macro-renamed while
//     that header is read, then redefined with the workload's values
//     (passed as -DSLREF_* by oracle/Makefile);
//   * `path`/`targetName` (dust_const.hpp:65-66) point at a two-sphere dummy
//     save written at load time, because the reference constructs its global
//     `Ball_group O(path, targetName, 0)` (ColliderSingleCore.cpp:33) from a
//     saved simulation before main runs;
//   * the reference's main() is renamed so the harness can export a C API;
//   * Ball_group's private members (its save loader) are made accessible to
//     the harness by compiling the reference headers with `private` defined
//     as `public`; every standard header the reference uses is included
//     first, so only the reference's own classes see that definition.
#include <algorithm>
#include <array>
#include <cassert>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <fstream>
#include <functional>
#include <iomanip>
#include <iosfwd>
#include <iostream>
#include <limits.h>
#include <numbers>
#include <random>
#include <sstream>
#include <string>
#include <type_traits>
#include <unistd.h>
using std::isnan;

#define G G_ref
#define Ha Ha_ref
#define u_s u_s_ref
#define u_r u_r_ref
#define cor cor_ref
#define h_min h_min_ref
#define density density_ref
#define path path_ref
#define targetName targetName_ref
#include "dust_const.hpp"
#undef G
#undef Ha
#undef u_s
#undef u_r
#undef cor
#undef h_min
#undef density
#undef path
#undef targetName

constexpr double G = SLREF_G;
constexpr double Ha = SLREF_HA;
constexpr double u_s = SLREF_US;
constexpr double u_r = SLREF_UR;
constexpr double cor = SLREF_COR;
constexpr double h_min = SLREF_HMIN;
constexpr double density = SLREF_DENSITY;

// Two far-apart heavy spheres in the reference's save format (11 columns per
// sphere, no trailing newline after the last row), so that the reference's
// continue-constructor has something to load.  Heavy masses make its
// collapse-speed loop (ball_group.hpp:302-314) end after one iteration.
static std::string slref_dummy_dir()
{
    char tmpl[] = "/tmp/slref_XXXXXX";
    const char* dir = mkdtemp(tmpl);
    if (!dir) { std::perror("slref: mkdtemp"); std::abort(); }
    const std::string d = std::string(dir) + "/";
    std::ofstream sim(d + "slref_dummy_simData.csv");
    sim << "x0,y0,z0,wx0,wy0,wz0,wmag0,vx0,vy0,vz0,bound0,x1,y1,z1,wx1,wy1,wz1,wmag1,vx1,vy1,vz1,bound1\n"
        << "1,0,0,0,0,0,0,0,0,0,0,-1,0,0,0,0,0,0,0,0,0,0";
    sim.close();
    std::ofstream con(d + "slref_dummy_constants.csv");
    con << "0.0001,1e10,1\n0.0001,1e10,1\n";
    con.close();
    std::cerr.setstate(std::ios::badbit);  // the reference's setup chatter
    return d;
}
std::string path = slref_dummy_dir();
std::string targetName = "slref_dummy_";

// The reference TU.  SLREF_COLLIDER_TU names another copy of it: the
// drop-in check (oracle/Makefile, target `adapter`) compiles the copy a
// maintainer would have after adding the GPU adapter
// (include/spacelab_sim_one_step_gpu.hpp) and defines SLREF_GPU_ADAPTER.
#ifndef SLREF_COLLIDER_TU
#define SLREF_COLLIDER_TU "ColliderSingleCore/ColliderSingleCore.cpp"
#endif
#define private public
#define main reference_main
#include SLREF_COLLIDER_TU
#undef main
#undef private

static void slref_take_energy(double* e)
{
    if (e) {
        e[0] = O.PE; e[1] = O.KE;
        e[2] = O.mom.x; e[3] = O.mom.y; e[4] = O.mom.z;
        e[5] = O.ang_mom.x; e[6] = O.ang_mom.y; e[7] = O.ang_mom.z;
    }
    // the reference's caller resets the totals after each write
    // (ColliderSingleCore.cpp:341-344)
    O.KE = 0; O.PE = 0; O.mom = {0, 0, 0}; O.ang_mom = {0, 0, 0};
    ballBuffer.str("");
}

extern "C" {

void slref_material(double* out)
{
    out[0] = G; out[1] = Ha; out[2] = u_s; out[3] = u_r; out[4] = h_min;
}

// Load a state into the reference's global Ball_group and run its initial
// force pass: distances := current distances, then sim_one_step(true) with
// dt = 0, which evaluates exactly the pair terms of init_conditions
// (ball_group.hpp:777-947) and leaves pos/vel/w unchanged.
int slref_init(int n, const double* pos, const double* vel, const double* w, const double* R,
               const double* m, const double* moi, double dt_, double kin_, double kout_, double* energy)
{
    if (n < 1) return 1;
    O = Ball_group(n);
    for (int i = 0; i < n; i++) {
        O.pos[i] = vec3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
        O.vel[i] = vec3(vel[3 * i], vel[3 * i + 1], vel[3 * i + 2]);
        O.w[i] = vec3(w[3 * i], w[3 * i + 1], w[3 * i + 2]);
        O.velh[i] = vec3(0, 0, 0); O.wh[i] = vec3(0, 0, 0);
        O.acc[i] = vec3(0, 0, 0); O.aacc[i] = vec3(0, 0, 0);
        O.R[i] = R[i]; O.m[i] = m[i]; O.moi[i] = moi[i];
    }
    for (int A = 1; A < n; A++)
        for (int B = 0; B < A; B++)
            O.distances[static_cast<long>(A) * (A - 1) / 2 + B] = (O.pos[B] - O.pos[A]).norm();
    O.KE = 0; O.PE = 0; O.mom = {0, 0, 0}; O.ang_mom = {0, 0, 0};
    kin = kin_; kout = kout_;
    dt = 0;
    sim_one_step(true);
    dt = dt_;
    slref_take_energy(energy);
    return 0;
}

// Resume a state inside the reference's global Ball_group after
// slref_init: pos/vel/w/acc/aacc as given, and `distances` from the
// positions of the previous step (ball_group.hpp:741; the reference stores
// exactly those pair distances at the end of each pass 2).  NULL pos_prev =
// pos.
int slref_resume(const double* pos, const double* vel, const double* w, const double* acc, const double* aacc,
                 const double* pos_prev)
{
    const int n = O.num_particles;
    if (n < 1) return 1;
    const double* prev = pos_prev ? pos_prev : pos;
    for (int i = 0; i < n; i++) {
        O.pos[i] = vec3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
        O.vel[i] = vec3(vel[3 * i], vel[3 * i + 1], vel[3 * i + 2]);
        O.w[i] = vec3(w[3 * i], w[3 * i + 1], w[3 * i + 2]);
        O.acc[i] = vec3(acc[3 * i], acc[3 * i + 1], acc[3 * i + 2]);
        O.aacc[i] = vec3(aacc[3 * i], aacc[3 * i + 1], aacc[3 * i + 2]);
    }
    for (int A = 1; A < n; A++) {
        const vec3 pa(prev[3 * A], prev[3 * A + 1], prev[3 * A + 2]);
        for (int B = 0; B < A; B++) {
            const vec3 pb(prev[3 * B], prev[3 * B + 1], prev[3 * B + 2]);
            O.distances[static_cast<long>(A) * (A - 1) / 2 + B] = (pb - pa).norm();
        }
    }
    O.KE = 0; O.PE = 0; O.mom = {0, 0, 0}; O.ang_mom = {0, 0, 0};
    return 0;
}

// The reference's own run: Ball_group::sim_init_write(prefix) (simData,
// constants and energy files with the state and totals of the initial force
// pass, ball_group.hpp:421-516), then sim_looper (ColliderSingleCore.cpp:
// 291-375) for steps 1..steps_-1 with a write step every skip_ steps, which
// appends the simData and energy rows.  Call after slref_init; init_energy
// are its totals.  With SLREF_GPU_ADAPTER the looper's steps run on the GPU
// through the adapter.  Returns the output prefix actually used (the writer
// prepends a counter when files of that name exist).
const char* slref_looper(const char* prefix, int steps_, int skip_, const double* init_energy)
{
    static std::string used;
    energyBuffer.precision(12);  // as the reference's main does (:42)
    ballBuffer.str("");
    energyBuffer.str("");
    O.PE = init_energy[0];
    O.KE = init_energy[1];
    O.mom = vec3(init_energy[2], init_energy[3], init_energy[4]);
    O.ang_mom = vec3(init_energy[5], init_energy[6], init_energy[7]);
    O.sim_init_write(prefix);
    O.KE = 0; O.PE = 0; O.mom = {0, 0, 0}; O.ang_mom = {0, 0, 0};
    simTimeElapsed = 0;
    steps = steps_;
    skip = skip_;
#ifdef SLREF_GPU_ADAPTER
    sl_gpu_begin();
#endif
    sim_looper();
#ifdef SLREF_GPU_ADAPTER
    sl_gpu_sync_host();
    sl_gpu_end();
#endif
    used = output_prefix;
    return used.c_str();
}

// One reference step; energy (8 doubles) is filled on write steps.
void slref_step(int write, double* energy)
{
    sim_one_step(write != 0);
    if (write) slref_take_energy(energy);
}

void slref_get(double* pos, double* vel, double* w, double* acc, double* aacc)
{
    for (int i = 0; i < O.num_particles; i++) {
        for (int c = 0; c < 3; c++) {
            if (pos) pos[3 * i + c] = O.pos[i][c];
            if (vel) vel[3 * i + c] = O.vel[i][c];
            if (w) w[3 * i + c] = O.w[i][c];
            if (acc) acc[3 * i + c] = O.acc[i][c];
            if (aacc) aacc[3 * i + c] = O.aacc[i][c];
        }
    }
}

// Load a save with the reference's own loader: Ball_group::loadSim =
// getLastLine + parseSimData + loadConsts (ball_group.hpp:1236-1247).
int slref_load_sim(const char* path, const char* name, int maxn, int* n, double* pos, double* vel, double* w,
                   double* R, double* m, double* moi)
{
    Ball_group g;
    g.loadSim(path, name);
    *n = g.num_particles;
    if (g.num_particles > maxn) return 1;
    for (int i = 0; i < g.num_particles; i++) {
        for (int c = 0; c < 3; c++) {
            pos[3 * i + c] = g.pos[i][c];
            vel[3 * i + c] = g.vel[i][c];
            w[3 * i + c] = g.w[i][c];
        }
        R[i] = g.R[i]; m[i] = g.m[i]; moi[i] = g.moi[i];
    }
    return 0;
}

// Write a save with the reference's own writer, Ball_group::sim_init_write
// (ball_group.hpp:421-516): simData header + one row, constants, energy.
int slref_write_sim(const char* prefix, int n, const double* pos, const double* vel, const double* w,
                    const double* R, const double* m, const double* moi)
{
    Ball_group g(n);
    for (int i = 0; i < n; i++) {
        g.pos[i] = vec3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
        g.vel[i] = vec3(vel[3 * i], vel[3 * i + 1], vel[3 * i + 2]);
        g.w[i] = vec3(w[3 * i], w[3 * i + 1], w[3 * i + 2]);
        g.R[i] = R[i]; g.m[i] = m[i]; g.moi[i] = moi[i];
    }
    g.sim_init_write(prefix);
    return 0;
}

}  // extern "C"
