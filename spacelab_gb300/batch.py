"""Batched projectile-target collisions (include/spacelab_batch.h).

``sample_collisions`` draws a sweep of collisions:

- target size N_t uniform in [64, 1600];
- projectile size N_p uniform in [8, N_t/2];
- impact speed log-uniform in [10, 1000] cm/s;
- impact parameter b uniform in [0, 1] x (R_t + R_p);
- coefficient of restitution uniform in [0.4, 0.8];
- friction mu uniform in [0.1, 0.5].

Each instance is built like the N=5000 aggregate collision: two seeded
clusters, the projectile 1.1 (R_t + R_p) away along x and b along y, opposite
kicks to zero momentum, target first, centre of mass at the origin. Its k
comes from the reference's formula at 1/50 of the impact speed (as the
N=5000 collision's 2 cm/s for 100 cm/s), and dt = contact time / 50.  The
projectile then travels ~12 radii in 3000 steps at any speed (dt scales as
1/speed), enough to reach the target from 1.1 (R_t + R_p), and a head-on
impact overlaps ~9% of a radius, below the reference's design overlap of
10% (maxOverlap, dust_const.hpp:31).

``BatchRun`` advances all instances in one persistent launch; ``run_per_instance``
is the comparison: the same instances one after another through the
single-system step.
"""
from __future__ import annotations

import ctypes
import time
from dataclasses import dataclass, field

import numpy as np

from . import _lib, configs
from ._lib import Material, check, dptr
from .ball_group import MODES, BallGroup, GpuStep


@dataclass
class Collision:
    n_t: int
    n_p: int
    speed: float
    b_frac: float
    cor: float
    mu: float
    seed: int
    group: BallGroup | None = None
    dt: float = 0.0
    kin: float = 0.0
    kout: float = 0.0
    info: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return self.n_t + self.n_p


def sample_collisions(count: int, seed: int, nt_range=(64, 1600), speed_range=(10.0, 1000.0), cor_range=(0.4, 0.8),
                      mu_range=(0.1, 0.5), build: bool = True, clearance: float | None = None,
                      k_speed_div: float = 50.0) -> list[Collision]:
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        n_t = int(rng.integers(nt_range[0], nt_range[1] + 1))
        n_p = int(rng.integers(8, max(8, n_t // 2) + 1))
        speed = float(np.exp(rng.uniform(np.log(speed_range[0]), np.log(speed_range[1]))))
        c = Collision(n_t, n_p, speed, float(rng.uniform(0, 1)), float(rng.uniform(*cor_range)),
                      float(rng.uniform(*mu_range)), int(rng.integers(1, 2 ** 62)))
        if build:
            build_instance(c, clearance, k_speed_div)
        out.append(c)
    return out


def cluster_seeds(c: Collision) -> tuple[int, int]:
    """Seeds of the target's and the projectile's cluster."""
    return c.seed, c.seed ^ 0x5DEECE66D


def build_instance(c: Collision, clearance: float | None = None, k_speed_div: float = 50.0) -> Collision:
    """Build the two clusters.  clearance None: centres 1.1 (R_t + R_p) apart
    along x; otherwise the bounding spheres are `clearance` sphere radii
    apart.  k from the reference formula at speed / k_speed_div."""
    if clearance is None:
        off_x = 1.1
    else:
        rt = configs.RADIUS * (c.n_t / configs.PHI) ** (1 / 3)
        rp = configs.RADIUS * (c.n_p / configs.PHI) ** (1 / 3)
        off_x = 1.0 + clearance * configs.RADIUS / (rt + rp)
    seed_t, seed_p = cluster_seeds(c)
    g = configs.build_collision(c.n_t, c.n_p, c.speed, off_x, c.b_frac, seed_t, seed_p)
    kin, kout, dt = configs.spring_and_dt(float(g.R.max()), float(g.m.min()), c.speed / k_speed_div,
                                          cor=c.cor * c.cor)
    c.group, c.kin, c.kout, c.dt = g, kin, kout, dt
    c.info.update({"off_x": off_x, "k_speed_div": k_speed_div})
    return c


def instance_material(c: Collision) -> Material:
    m = configs.dust_material()
    m.u_s = c.mu
    return m


class BatchRun:
    """All instances of a sweep in one device batch."""

    def __init__(self, cols: list[Collision], mode: str = "exact", steps: int = 3000, skip: int = 100):
        self.lib = _lib.lib()
        self.cols = cols
        self.mode = mode
        self.steps, self.skip = steps, skip
        counts = np.array([c.n for c in cols], dtype=np.int32)
        self.counts = counts
        self.offsets = np.concatenate([[0], np.cumsum(counts)[:-1]]).astype(np.int64)
        self.total = int(counts.sum())
        mat = configs.dust_material()
        h = ctypes.c_void_p()
        check(self.lib.sl_batch_create(len(cols), counts.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                       ctypes.byref(mat), MODES[mode], steps, skip, ctypes.byref(h)), "sl_batch_create")
        self.h = h
        cat = lambda k: np.ascontiguousarray(np.concatenate([getattr(c.group, k) for c in cols]))  # noqa: E731
        pos, vel, w = (cat(k).reshape(-1) for k in ("pos", "vel", "w"))
        R, m, moi = (cat(k) for k in ("R", "m", "moi"))
        par = [np.array([getattr(c, k) for c in cols], dtype=np.float64) for k in ("dt", "kin", "kout")]
        u_s = np.array([c.mu for c in cols], dtype=np.float64)
        check(self.lib.sl_batch_upload(self.h, *[dptr(a) for a in (pos, vel, w, R, m, moi, *par, u_s)]),
              "sl_batch_upload")

    def close(self):
        if self.h:
            self.lib.sl_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_shape(self, tile: int, threads: int):
        check(self.lib.sl_batch_set_shape(self.h, tile, threads), "sl_batch_set_shape")

    def shape(self) -> tuple[int, int, int]:
        t, th, b = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        check(self.lib.sl_batch_shape(self.h, ctypes.byref(t), ctypes.byref(th), ctypes.byref(b)), "sl_batch_shape")
        return t.value, th.value, b.value

    def autotune(self, sample_steps: int = 3) -> dict:
        t, th = ctypes.c_int(), ctypes.c_int()
        times = np.zeros(12)
        check(self.lib.sl_batch_autotune(self.h, sample_steps, ctypes.byref(t), ctypes.byref(th), dptr(times)),
              "sl_batch_autotune")
        grid = {(f"tile{tl}" if tl else "pairtiles") + f"_threads{thr}": float(times[3 * i + j])
                for i, tl in enumerate((32, 64, 128, 0))
                for j, thr in enumerate((128, 256, 512) if tl == 0 and self.mode == "mixed_df" else (64, 128, 256))
                if times[3 * i + j] >= 0}
        return {"tile": t.value, "threads": th.value, "times_ms": grid}

    def run(self, first_step: int = 1, nsteps: int | None = None, do_init: bool = True) -> float:
        nsteps = self.steps if nsteps is None else nsteps
        t0 = time.perf_counter()
        check(self.lib.sl_batch_run(self.h, first_step, nsteps, int(do_init)), "sl_batch_run")
        return time.perf_counter() - t0

    def state(self) -> dict:
        arr = {k: np.zeros(3 * self.total) for k in ("pos", "vel", "w", "acc", "aacc")}
        check(self.lib.sl_batch_download(self.h, *[dptr(arr[k]) for k in ("pos", "vel", "w", "acc", "aacc")]),
              "sl_batch_download")
        return {k: v.reshape(-1, 3) for k, v in arr.items()}

    def instance_state(self, st: dict, i: int) -> dict:
        a, b = int(self.offsets[i]), int(self.offsets[i] + self.counts[i])
        return {k: v[a:b] for k, v in st.items()}

    def energy(self) -> np.ndarray:
        nrec = ctypes.c_int()
        check(self.lib.sl_batch_energy(self.h, None, ctypes.byref(nrec)), "sl_batch_energy")
        e = np.zeros(len(self.cols) * nrec.value * 8)
        check(self.lib.sl_batch_energy(self.h, dptr(e), ctypes.byref(nrec)), "sl_batch_energy")
        return e.reshape(len(self.cols), nrec.value, 8)

    def status(self) -> np.ndarray:
        s = np.zeros(len(self.cols), dtype=np.uint32)
        check(self.lib.sl_batch_status(self.h, s.ctypes.data_as(ctypes.POINTER(ctypes.c_uint))), "sl_batch_status")
        return s


def stratified_indices(cols: list[Collision], k: int) -> np.ndarray:
    """k collisions at evenly spaced quantiles of the sphere count (the
    middle of k equal-count strata of the size-sorted sweep), so that a
    per-instance baseline timed on them and scaled by len(cols) / k
    estimates the whole sweep's time without size bias."""
    order = np.argsort([c.n for c in cols], kind="stable")
    k = min(k, len(cols))
    pick = ((np.arange(k) + 0.5) * len(cols) / k).astype(int)
    return order[pick]


def made_contact(energy: np.ndarray, frac: float = 1e-3) -> np.ndarray:
    """Per instance, whether its clusters touched: restitution and friction
    dissipate energy only in contact, so E = PE + KE falling by more than
    `frac` of the initial kinetic energy marks a contact.  energy is
    [ninst][nrec][8] (BatchRun.energy)."""
    E = energy[:, :, 0] + energy[:, :, 1]
    return (E[:, 0] - E[:, -1]) > frac * energy[:, 0, 1]


def run_per_instance(cols: list[Collision], steps: int, skip: int, mode: str = "exact") -> tuple[float, list]:
    """The same collisions one after another through the single-system path
    (sl_run per instance); returns (seconds, final states)."""
    states = []
    t0 = time.perf_counter()
    for c in cols:
        with GpuStep(c.group.copy(), instance_material(c), mode) as s:
            s.set_scalars(c.dt, c.kin, c.kout)
            s.init_conditions()
            s.sim_looper(steps=steps + 1, skip=skip)
            g = s.download()
            states.append({k: getattr(g, k).copy() for k in ("pos", "vel", "w", "acc", "aacc")})
    return time.perf_counter() - t0, states


def run_per_instance_steps(cols: list[Collision], steps: int, skip: int, mode: str = "exact") -> float:
    """The same collisions one after another, one sim_one_step call (sl_step
    with its host round trip) per step: the drop-in used step by step."""
    t0 = time.perf_counter()
    for c in cols:
        with GpuStep(c.group.copy(), instance_material(c), mode) as s:
            s.set_scalars(c.dt, c.kin, c.kout)
            s.init_conditions()
            for step in range(1, steps + 1):
                s.sim_one_step(step % skip == 0)
    return time.perf_counter() - t0
