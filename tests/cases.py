"""Seeded input cases for the parity tests.

`contact_case` packs spheres on a jittered cubic lattice at a spacing below
the mean contact distance, so that about half of the neighbour pairs start
in contact, with fast random velocities and spins: every branch of the
reference's pair loop (contact and non-contact, kin/kout, sliding and
rolling friction, torques, h < h_min) is exercised within a few steps.
"""
from __future__ import annotations

import numpy as np

RADIUS = 1e-4
DENSITY = 1.70
MATERIAL = dict(G=6.674e-8, Ha=4e-13, u_s=0.3, u_r=1e-5, h_min=1e-5)


def material():
    from spacelab_gb300._lib import Material
    return Material(**MATERIAL)


class OracleMaterial:
    def __init__(self):
        for k, v in MATERIAL.items():
            setattr(self, k, v)


def contact_case(n: int, seed: int, spacing: float = 1.97, vel_sigma: float = 50.0, w_sigma: float = 2e5,
                 r_spread: float = 0.1, k_speed: float = 100.0) -> dict:
    rng = np.random.default_rng(seed)
    side = max(1, int(np.ceil(n ** (1 / 3))))
    g = np.stack(np.meshgrid(*[np.arange(side)] * 3, indexing="ij"), -1).reshape(-1, 3)[:n].astype(np.float64)
    pos = g * spacing * RADIUS + rng.normal(0.0, 0.02 * RADIUS, (n, 3))
    pos -= pos.mean(axis=0)
    R = RADIUS * rng.uniform(1 - r_spread, 1 + r_spread, n)
    m = DENSITY * 4.0 / 3.0 * np.pi * R ** 3
    moi = 0.4 * m * R * R
    vel = rng.normal(0.0, vel_sigma, (n, 3))
    w = rng.normal(0.0, w_sigma, (n, 3))
    kconsts = 3e3 * (4.0 / 3.0 * np.pi * DENSITY) / 0.01
    kin = kconsts * R.max() * k_speed ** 2
    kout = 0.4096 * kin
    dt = np.pi * np.sqrt(m.min() / (2 * kin)) / 50
    return dict(pos=pos, vel=vel, w=w, R=R, m=m, moi=moi, dt=float(dt), kin=float(kin), kout=float(kout))


def two_sphere_case(gap_fraction: float) -> dict:
    """Two unit spheres on the x axis; gap_fraction < 0 overlaps."""
    R = np.array([RADIUS, RADIUS])
    d = 2 * RADIUS * (1 + gap_fraction)
    pos = np.array([[-d / 2, 0.0, 0.0], [d / 2, 0.0, 0.0]])
    vel = np.array([[10.0, 1.0, 0.0], [-10.0, 0.0, 2.0]])
    w = np.array([[0.0, 0.0, 1e4], [1e3, 0.0, 0.0]])
    m = DENSITY * 4.0 / 3.0 * np.pi * R ** 3
    moi = 0.4 * m * R * R
    kin = 3e3 * (4.0 / 3.0 * np.pi * DENSITY) / 0.01 * RADIUS * 100.0 ** 2
    return dict(pos=pos, vel=vel, w=w, R=R, m=m, moi=moi, dt=float(np.pi * np.sqrt(m[0] / (2 * kin)) / 50),
                kin=float(kin), kout=float(0.4096 * kin))


def write_schedule(step: int, every: int) -> bool:
    return step % every == 0


GOLDEN_CASES = [
    # (name, n, seed, steps, write_every)
    ("contact_n2", 2, 11, 100, 10),
    ("contact_n33", 33, 12, 100, 10),
    ("contact_n64", 64, 13, 100, 10),
    ("contact_n257", 257, 14, 100, 10),
]
GOLDEN_CHECKPOINTS = (1, 10, 100)


def golden_case_inputs(name: str) -> dict:
    for nm, n, seed, _, _ in GOLDEN_CASES:
        if nm == name:
            if n == 2:
                return two_sphere_case(-0.03)
            return contact_case(n, seed)
    raise KeyError(name)
