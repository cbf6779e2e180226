"""Workloads of the dust-aggregate benchmarks, built by the seeded C++
builder (include/spacelab_host.h).

Material: G = 6.674e-8, Hamaker A = 4e-13 erg, mu = 0.3, rolling mu = 1e-5
(the reference's u_r, dust_const.hpp:24), h_min = 0.1 a, sphere radius
a = 1e-4 cm, density 1.70 g/cm^3, coefficient of restitution e = 0.64
(kout = e^2 kin, the reference's `cor` semantics, ball_group.hpp:1317,1231).
Spring constant from the reference's formula kin = kConsts r_max v^2
(ball_group.hpp:1316) at a stated speed v; dt = contact time / 50.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from ._lib import Material, dptr
from .ball_group import BallGroup

RADIUS = 1e-4
DENSITY = 1.70
PHI = 0.3
COR_E = 0.64
COR = COR_E * COR_E
STEPS_PER_CONTACT = 50.0


def dust_material() -> Material:
    return Material(G=6.674e-8, Ha=4e-13, u_s=0.3, u_r=1e-5, h_min=0.1 * RADIUS)


@dataclass
class Workload:
    name: str
    group: BallGroup
    dt: float
    kin: float
    kout: float
    steps: int
    skip: int
    material: Material = field(default_factory=dust_material)
    info: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return self.group.num_particles

    @property
    def pairs_per_step(self) -> int:
        return self.n * (self.n - 1) // 2


def spring_and_dt(r_max: float, m_min: float, speed: float, cor: float = COR) -> tuple[float, float, float]:
    kin, kout, dt = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    rc = _lib.lib().slh_spring_and_dt(r_max, m_min, speed, DENSITY, cor, STEPS_PER_CONTACT, ctypes.byref(kin),
                                      ctypes.byref(kout), ctypes.byref(dt))
    if rc != 0:
        raise ValueError("bad spring/dt arguments")
    return kin.value, kout.value, dt.value


def build_cluster(n: int, seed: int, sigma_v: float, sigma_ln: float = 0.0, clip=(0.5, 2.0),
                  radius: float = RADIUS, phi: float = PHI) -> BallGroup:
    g = BallGroup(n)
    pos, vel, w = (np.zeros(3 * n) for _ in range(3))
    R, m, moi = (np.zeros(n) for _ in range(3))
    rc = _lib.lib().slh_build_cluster(n, radius, sigma_ln, clip[0], clip[1], DENSITY, phi, sigma_v, seed,
                                      dptr(pos), dptr(vel), dptr(w), dptr(R), dptr(m), dptr(moi))
    if rc != 0:
        raise RuntimeError(f"slh_build_cluster failed ({rc})")
    g.pos[:] = pos.reshape(-1, 3); g.vel[:] = vel.reshape(-1, 3); g.w[:] = w.reshape(-1, 3)
    g.R[:] = R; g.m[:] = m; g.moi[:] = moi
    return g


def build_collision(n_t: int, n_p: int, speed: float, off_x: float, off_y: float, seed_t: int, seed_p: int,
                    sigma_v: float = 1e-3, radius: float = RADIUS, phi: float = PHI) -> BallGroup:
    n = n_t + n_p
    g = BallGroup(n)
    pos, vel, w = (np.zeros(3 * n) for _ in range(3))
    R, m, moi = (np.zeros(n) for _ in range(3))
    rc = _lib.lib().slh_build_collision(n_t, n_p, radius, DENSITY, phi, sigma_v, speed, off_x, off_y, seed_t,
                                        seed_p, dptr(pos), dptr(vel), dptr(w), dptr(R), dptr(m), dptr(moi))
    if rc != 0:
        raise RuntimeError(f"slh_build_collision failed ({rc})")
    g.pos[:] = pos.reshape(-1, 3); g.vel[:] = vel.reshape(-1, 3); g.w[:] = w.reshape(-1, 3)
    g.R[:] = R; g.m[:] = m; g.moi[:] = moi
    return g


def dust_cluster_1000(seed: int = 1000) -> Workload:
    """1000 monodisperse spheres, sigma_v = 1e-3 cm/s, 2000 steps, energy
    every 100; k at v = 1 cm/s (order of the vdW sticking speed)."""
    g = build_cluster(1000, seed, sigma_v=1e-3)
    kin, kout, dt = spring_and_dt(float(g.R.max()), float(g.m.min()), 1.0)
    return Workload("dust_cluster_n1000", g, dt, kin, kout, steps=2000, skip=100,
                    info={"seed": seed, "k_speed_cm_s": 1.0})


def aggregate_collision_5000(seed_t: int = 4000, seed_p: int = 1001, k_speed: float = 2.0) -> Workload:
    """4000-sphere target + 1000-sphere projectile, 1.1 (Rt+Rp) apart along x,
    impact parameter 0.3 (Rt+Rp) along y, 100 cm/s relative speed, 5000
    steps, energy every 100.

    k from the reference formula kConsts r_max v^2 at v = k_speed.  The
    workload fixes the geometry, the speed and the step count, and asks the
    contact time to span 50 steps, which leaves k to choose; it must be soft
    enough that the clusters meet inside the 5000 steps (the projectile
    travels ~6 radii before the first contact) and stiff enough that the
    100 cm/s impact stays below the reference's design overlap of 10% of a
    radius (maxOverlap, dust_const.hpp:31).  At 2 cm/s the impact overlaps
    ~6.5% of a radius and dt = 4.1e-9 s, so the projectile covers ~20 radii
    in the 5000 steps."""
    g = build_collision(4000, 1000, 100.0, 1.1, 0.3, seed_t, seed_p)
    kin, kout, dt = spring_and_dt(float(g.R.max()), float(g.m.min()), k_speed)
    return Workload("aggregate_collision_n5000", g, dt, kin, kout, steps=5000, skip=100,
                    info={"seed_target": seed_t, "seed_projectile": seed_p, "speed_cm_s": 100.0,
                          "k_speed_cm_s": k_speed})


def polydisperse_cluster_20000(seed: int = 20000) -> Workload:
    """20000 spheres, lognormal radii (median 1e-4, sigma_ln 0.2, clipped to
    [0.5, 2] x median), phi = 0.3, sigma_v = 1e-2 cm/s, 10000 steps."""
    g = build_cluster(20000, seed, sigma_v=1e-2, sigma_ln=0.2)
    kin, kout, dt = spring_and_dt(float(g.R.max()), float(g.m.min()), 1.0)
    return Workload("polydisperse_cluster_n20000", g, dt, kin, kout, steps=10000, skip=100,
                    info={"seed": seed, "k_speed_cm_s": 1.0})
