/*
 * spacelab_host.h -- C ABI of the host-side setup that surrounds the GPU
 * step (libspacelab_gb300.so): seeded cluster building, the spring/time-step
 * recipe and the reference's centring.  Arrays are the reference's layouts:
 * vec3[n] (3n doubles, x y z per sphere) and double[n].
 *
 * These replace the reference's generation and setup code, which draws from
 * std::random_device and is not reproducible (Utils.hpp:28-29,166-171;
 * ball_group.hpp:1126-1233).  All random numbers come from a seeded
 * xoshiro256** stream and only IEEE basic operations (+ - * / sqrt), so a
 * seed gives the same bits on every host.
 */
#ifndef SPACELAB_HOST_H
#define SPACELAB_HOST_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* One cluster, Generator-style: radii lognormal with the given median and
 * sigma_ln, clipped to [clip_lo, clip_hi] x median (sigma_ln = 0 gives
 * monodisperse spheres), placed by random sequential addition without
 * overlap, centres uniform in a sphere of radius
 * median * (n / phi)^(1/3); velocities Gaussian with sigma_v per component;
 * w = 0; m = rho 4/3 pi R^3; moi = 0.4 m R^2 (ball_group.hpp:573).
 * The cluster is shifted to its centre of mass (ball_group.hpp:542-547).
 * Returns 0, or 1 on bad arguments, 2 if placement failed. */
int slh_build_cluster(int n, double median_radius, double sigma_ln, double clip_lo, double clip_hi,
                      double rho, double phi, double sigma_v, uint64_t seed, double* pos, double* vel,
                      double* w, double* R, double* m, double* moi);

/* Projectile-target collision of two such monodisperse clusters
 * (ball_group.hpp:1368-1442 semantics): the projectile is offset by
 * (off_x, off_y, 0) x (Rt + Rp), Rt/Rp the clusters' placement radii; it is
 * kicked by -speed along x and the target by +(m_p/m_t) speed so the total
 * momentum is zero (ball_group.hpp:1415-1425); target spheres come first
 * (ball_group.hpp:1435-1436) and the merged system is shifted to its centre
 * of mass.  Output arrays hold n_t + n_p spheres. */
int slh_build_collision(int n_t, int n_p, double radius, double rho, double phi, double sigma_v,
                        double speed, double off_x, double off_y, uint64_t seed_t, uint64_t seed_p,
                        double* pos, double* vel, double* w, double* R, double* m, double* moi);

/* Radii of gyration of `count` monodisperse clusters, each built exactly as
 * slh_build_collision builds its target and its projectile (slh_build_cluster
 * with sigma_ln = 0 and the velocity spread 1e-3 cm/s, which does not move
 * the spheres): cluster k has n[k] spheres of `radius` from seed[k].  rg[k]
 * gets its radius of gyration (-1 if it could not be built).  `threads` host
 * threads (< 1: all).  No counterpart in the reference: it gives a
 * collision sweep its clusters' measured radii of gyration without keeping
 * the clusters.  Returns 0, 1 on bad arguments, 2 if a cluster failed. */
int slh_cluster_rg(int count, const int* n, const uint64_t* seed, double radius, double rho, double phi,
                   int threads, double* rg);

/* Spring constants and time step: kin = kConsts r_max v^2 with
 * kConsts = 3e3 (4/3 pi rho) / maxOverlap^2, maxOverlap = 0.1
 * (ball_group.hpp:1316, dust_const.hpp:30-35); kout = cor kin
 * (ball_group.hpp:1317; cor = e^2 for a coefficient of restitution e);
 * dt = pi sqrt(m_min / (2 kin)) / steps_per_contact. */
int slh_spring_and_dt(double r_max, double m_min, double speed, double rho, double cor,
                      double steps_per_contact, double* kin, double* kout, double* dt);

/* Shift positions so the mass-weighted centre is at the origin, with the
 * reference's operation order (ball_group.hpp:519-547). */
int slh_to_origin(int n, double* pos, const double* m);

/* --- the reference's files (return 0, 1 bad argument, 3 I/O error, 4 format error) ---
 * Writers produce the reference's formats: simData.csv (header
 * ball_group.hpp:463-472; rows ColliderSingleCore.cpp:259,268-280),
 * energy.csv (ball_group.hpp:462, ColliderSingleCore.cpp:335-338) and
 * constants.csv (ball_group.hpp:475-477), numbers as printf("%.*g",
 * precision): 6 is what the reference writes (lossy), 17 round-trips. */
int slh_write_simdata_header(const char* path, int n);
int slh_append_simdata_row(const char* path, int n, const double* pos, const double* w, const double* vel,
                           int precision);
int slh_write_energy_header(const char* path);
int slh_append_energy_row(const char* path, double time, double PE, double KE, double p, double L, int precision);
int slh_write_constants(const char* path, int n, const double* R, const double* m, const double* moi,
                        int precision);
/* Continue from a save (getLastLine/parseSimData/loadConsts,
 * ball_group.hpp:979-1077): the state is the last row of simData.csv. */
int slh_count_last_state(const char* simdata_path, int* n);
int slh_read_last_state(const char* simdata_path, int n, double* pos, double* vel, double* w);
int slh_read_constants(const char* constants_path, int n, double* R, double* m, double* moi);
/* Exact binary checkpoint (no counterpart in the reference, whose CSV save
 * keeps 6 digits and drops acc/aacc and the previous-step distances): the
 * full state including previous positions, so that a resumed run
 * (sl_upload_resume) continues bit for bit. */
int slh_write_checkpoint(const char* path, int n, const double* pos, const double* vel, const double* w,
                         const double* acc, const double* aacc, const double* pos_prev, const double* R,
                         const double* m, const double* moi, double dt, double kin, double kout, double sim_time,
                         long long step);
int slh_read_checkpoint_header(const char* path, int* n, double* dt, double* kin, double* kout, double* sim_time,
                               long long* step);
int slh_read_checkpoint(const char* path, int n, double* pos, double* vel, double* w, double* acc, double* aacc,
                        double* pos_prev, double* R, double* m, double* moi);

/* Outcome of a projectile-target collision from its final state (no
 * counterpart in the reference, whose `bound` column is always 0,
 * ball_group.hpp:496,502): connected components of spheres whose surface
 * gap is below bond_gap; largest_fraction = mass of the heaviest component /
 * total mass; stuck_fraction = projectile mass (spheres n_t..n-1) in it /
 * projectile mass; rg = its radius of gyration; n_components = count. */
int slh_collision_outcome(int n, int n_t, const double* pos, const double* R, const double* m, double bond_gap,
                          double* largest_fraction, double* stuck_fraction, double* rg, int* n_components);
/* Mass-weighted radius of gyration of a cluster. */
int slh_radius_of_gyration(int n, const double* pos, const double* m, double* rg);

/* Deterministic primitives, exported so tests can pin them. */
double slh_log(double x);
double slh_exp(double x);
uint64_t slh_rng_next(uint64_t* state4);

#ifdef __cplusplus
}
#endif
#endif /* SPACELAB_HOST_H */
