"""The reference-facing host interface: a Ball_group-shaped state and the GPU
drop-in for its step functions.

Reference interface mirrored here (paths inside the SpaceLab project):
  * ``Ball_group`` public arrays pos, vel, w, acc, aacc (vec3[n]) and R, m,
    moi (double[n]), totals PE, KE, mom, ang_mom   -- ball_group.hpp:18-53
  * ``sim_one_step(write_step)``                  -- ColliderSingleCore.cpp:78-288
  * ``sim_looper()``                              -- ColliderSingleCore.cpp:291-384
  * ``init_conditions()``                         -- ball_group.hpp:777-947
  * globals ``dt``, ``kin``, ``kout``             -- dust_const.hpp:51-53

As in the reference, the totals of a write step are *added* to the group's
PE/KE/mom/ang_mom and the looper resets them after recording an energy row
(ColliderSingleCore.cpp:333-344).  Errors raise SpaceLabError instead of the
reference's exit(EXIT_FAILURE).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import Energy, Material, SpaceLabError, check, dptr

# "mixed": FP32 force/torque arithmetic with FP64 displacements, close-pair
# overlaps and accumulation; "mixed_df": the double-float variant
MODES = {"exact": _lib.SL_MODE_EXACT, "mixed": _lib.SL_MODE_MIXED, "mixed_df": _lib.SL_MODE_MIXED_DF}


class BallGroup:
    """Ball_group's public state (ball_group.hpp:21-53) as numpy arrays."""

    def __init__(self, n: int):
        if n < 1:
            raise ValueError("a Ball_group needs at least one sphere")
        self.num_particles = int(n)
        self.pos = np.zeros((n, 3))
        self.vel = np.zeros((n, 3))
        self.w = np.zeros((n, 3))
        self.acc = np.zeros((n, 3))
        self.aacc = np.zeros((n, 3))
        self.R = np.ones(n)
        self.m = np.ones(n)
        self.moi = 0.4 * self.m * self.R * self.R  # calc_moi, ball_group.hpp:573
        self.PE = 0.0
        self.KE = 0.0
        self.mom = np.zeros(3)
        self.ang_mom = np.zeros(3)

    @classmethod
    def from_arrays(cls, pos, vel, w, R, m, moi) -> "BallGroup":
        g = cls(len(R))
        g.pos[:] = np.asarray(pos, dtype=np.float64).reshape(-1, 3)
        g.vel[:] = np.asarray(vel, dtype=np.float64).reshape(-1, 3)
        g.w[:] = np.asarray(w, dtype=np.float64).reshape(-1, 3)
        g.R[:] = R
        g.m[:] = m
        g.moi[:] = moi
        return g

    def copy(self) -> "BallGroup":
        g = BallGroup(self.num_particles)
        for k in ("pos", "vel", "w", "acc", "aacc", "R", "m", "moi", "mom", "ang_mom"):
            getattr(g, k)[:] = getattr(self, k)
        g.PE, g.KE = self.PE, self.KE
        return g

    def get_mass(self) -> float:
        """getMass, ball_group.hpp:1117-1124 (sequential sum)."""
        total = 0.0
        for mi in self.m:
            total += float(mi)
        return total

    def zero_totals(self) -> None:
        """The looper's reset after a write (ColliderSingleCore.cpp:341-344)."""
        self.PE = 0.0
        self.KE = 0.0
        self.mom[:] = 0.0
        self.ang_mom[:] = 0.0

    def add_totals(self, e: Energy) -> None:
        self.PE += e.PE
        self.KE += e.KE
        self.mom += np.array(e.mom[:])
        self.ang_mom += np.array(e.ang_mom[:])


@dataclass
class EnergyRow:
    """One row of the reference's energy.csv: Time,PE,KE,E,p,L
    (ball_group.hpp:462, ColliderSingleCore.cpp:335-338)."""

    time: float
    PE: float
    KE: float
    E: float
    p: float
    L: float


class GpuStep:
    """Device-resident drop-in for sim_one_step / sim_looper on one group.

    The group's arrays are uploaded once; the device copy is authoritative
    until ``download()`` writes it back into the group.
    """

    def __init__(self, group: BallGroup, material: Material, mode: str = "exact"):
        self._lib = _lib.lib()
        self.group = group
        self.material = material
        self.mode = mode
        self.dt = self.kin = self.kout = 0.0
        self.sim_time_elapsed = 0.0
        h = ctypes.c_void_p()
        check(self._lib.sl_create(group.num_particles, ctypes.byref(material), MODES[mode], ctypes.byref(h)),
              "sl_create")
        self._h = h
        self.upload()

    # -- lifetime -----------------------------------------------------------
    def close(self) -> None:
        if self._h:
            self._lib.sl_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self):
        return self._h

    # -- state transfer -----------------------------------------------------
    def upload(self) -> None:
        g = self.group
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (g.pos, g.vel, g.w, g.R, g.m, g.moi)]
        check(self._lib.sl_upload(self._h, *[dptr(a) for a in arrs]), "sl_upload")

    def upload_resume(self, pos_prev: np.ndarray | None = None) -> None:
        g = self.group
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (g.pos, g.vel, g.w, g.acc, g.aacc)]
        prev = None if pos_prev is None else np.ascontiguousarray(pos_prev, dtype=np.float64)
        check(self._lib.sl_upload_resume(self._h, *[dptr(a) for a in arrs], dptr(prev)), "sl_upload_resume")

    def download(self) -> BallGroup:
        g = self.group
        check(self._lib.sl_download(self._h, dptr(g.pos), dptr(g.vel), dptr(g.w), dptr(g.acc), dptr(g.aacc)),
              "sl_download")
        return g

    def set_scalars(self, dt: float, kin: float, kout: float) -> None:
        check(self._lib.sl_set_scalars(self._h, dt, kin, kout), "sl_set_scalars")
        self.dt, self.kin, self.kout = float(dt), float(kin), float(kout)

    # -- the hot path -------------------------------------------------------
    def init_conditions(self) -> Energy:
        """Initial forces and totals (ball_group.hpp:777-947); the totals are
        added to the group like the reference's init_conditions does."""
        e = Energy()
        check(self._lib.sl_init_forces(self._h, ctypes.byref(e)), "sl_init_forces")
        self.group.add_totals(e)
        return e

    def sim_one_step(self, write_step: bool) -> Energy | None:
        """One step (ColliderSingleCore.cpp:78-288); on write steps the totals
        are added to the group's PE/KE/mom/ang_mom."""
        e = Energy()
        check(self._lib.sl_step(self._h, 1, int(bool(write_step)), ctypes.byref(e)), "sl_step")
        if write_step:
            self.group.add_totals(e)
            return e
        return None

    def sim_one_step_host(self, write_step: bool) -> Energy | None:
        """One step on the state held in the group's host arrays
        (sl_step_host): they are read, stepped and overwritten in place; on
        write steps the totals are added to the group's PE/KE/mom/ang_mom."""
        g = self.group
        e = Energy()
        check(self._lib.sl_step_host(self._h, dptr(g.pos), dptr(g.vel), dptr(g.w), dptr(g.acc), dptr(g.aacc),
                                     int(bool(write_step)), ctypes.byref(e)), "sl_step_host")
        if write_step:
            g.add_totals(e)
            return e
        return None

    def step(self, nsteps: int, write_last: bool = False) -> Energy | None:
        e = Energy()
        check(self._lib.sl_step(self._h, int(nsteps), int(bool(write_last)), ctypes.byref(e)), "sl_step")
        return e if write_last else None

    def sim_looper(self, steps: int, skip: int, first_step: int = 1) -> list[EnergyRow]:
        """sim_looper (ColliderSingleCore.cpp:291-375): steps first_step ..
        steps-1, a write step whenever step % skip == 0; returns the energy
        rows the reference would append to energy.csv."""
        if skip < 1:
            raise SpaceLabError(_lib.SL_ERR_ARG, "sim_looper", "SKIP NOT SET")
        nwrites = sum(1 for s in range(first_step, steps) if s % skip == 0)
        rows = (Energy * max(1, nwrites))()
        nrows = ctypes.c_int(0)
        check(self._lib.sl_run(self._h, first_step, steps, skip, rows, nwrites, ctypes.byref(nrows)), "sl_run")
        out = []
        for k in range(nrows.value):
            e = rows[k]
            self.sim_time_elapsed += self.dt * skip  # :304
            p = float(np.linalg.norm(e.mom[:]))
            L = float(np.linalg.norm(e.ang_mom[:]))
            out.append(EnergyRow(self.sim_time_elapsed, e.PE, e.KE, e.PE + e.KE, p, L))
        return out

    def contacts(self) -> np.ndarray:
        """(A, B) contact pairs of the last force pass, reference loop order."""
        count = ctypes.c_long(0)
        check(self._lib.sl_contacts(self._h, None, 0, ctypes.byref(count)), "sl_contacts")
        buf = np.zeros(2 * max(1, count.value), dtype=np.int32)
        check(self._lib.sl_contacts(self._h, buf.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), count.value,
                                    ctypes.byref(count)), "sl_contacts")
        return buf[: 2 * count.value].reshape(-1, 2)

    def stream_ptr(self) -> int:
        return int(self._lib.sl_stream(self._h) or 0)

    def set_overlap(self, enable: bool) -> None:
        """Exact mode: pipeline the row sums with the pair phases (default off)."""
        check(self._lib.sl_set_overlap(self._h, int(enable)), "sl_set_overlap")

    def set_rowsum(self, method: str) -> None:
        """Exact mode: "fp64" (default) adds each row's FP64 terms on the FP64
        unit, "int" exactly on the integer pipe; the sums are identical."""
        code = {"int": 0, "fp64": 1}[method]
        check(self._lib.sl_set_rowsum(self._h, code), "sl_set_rowsum")

    def step_launches(self, write: bool) -> int:
        """Kernel launches of one step."""
        c = ctypes.c_int()
        check(self._lib.sl_step_launches(self._h, int(write), ctypes.byref(c)), "sl_step_launches")
        return c.value

    def pair_kernel(self) -> str:
        """Name of the pair kernel this handle's steps launch."""
        c = ctypes.c_char_p()
        check(self._lib.sl_pair_kernel(self._h, ctypes.byref(c)), "sl_pair_kernel")
        return c.value.decode()

    def kernel_timing(self, enable: bool) -> None:
        check(self._lib.sl_kernel_timing(self._h, int(enable)), "sl_kernel_timing")

    def kernel_times(self, reset: bool = True) -> tuple[float, float, int]:
        a, b, n = ctypes.c_double(), ctypes.c_double(), ctypes.c_long()
        check(self._lib.sl_kernel_times(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(n), int(reset)),
              "sl_kernel_times")
        return a.value, b.value, n.value

    def device_bytes(self) -> int:
        b = ctypes.c_uint64()
        check(self._lib.sl_device_bytes(self._h, ctypes.byref(b)), "sl_device_bytes")
        return b.value
