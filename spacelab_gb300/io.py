"""The reference's save files and an exact checkpoint, from Python.

``SimWriter`` mirrors sim_init_write plus the looper's periodic writes
(ball_group.hpp:421-516; ColliderSingleCore.cpp:268-280, 333-370):
<prefix>simData.csv, <prefix>energy.csv, <prefix>constants.csv.
``load_continue`` mirrors the reference's continue constructor's loading
(sim_continue -> loadSim, ball_group.hpp:1236-1247, 1352-1364).
``save_checkpoint`` / ``load_checkpoint`` keep the full state bit for bit.
"""
from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np

from . import _lib
from ._lib import dptr
from .ball_group import BallGroup, EnergyRow

REFERENCE_PRECISION = 6      # the reference writes simData/constants with ostream defaults
ENERGY_PRECISION = 12        # energyBuffer.precision(12), ColliderSingleCore.cpp:42


def _check(rc: int, what: str) -> None:
    if rc != 0:
        raise OSError(f"{what} failed (code {rc})")


def _b(p) -> bytes:
    return str(p).encode()


class SimWriter:
    """Writes a run in the reference's three-file format."""

    def __init__(self, prefix: str | Path, group: BallGroup, precision: int = REFERENCE_PRECISION):
        self.prefix = str(prefix)
        self.precision = precision
        self.n = group.num_particles
        lib = _lib.lib()
        _check(lib.slh_write_simdata_header(_b(self.simdata), self.n), "simData header")
        _check(lib.slh_write_energy_header(_b(self.energy)), "energy header")
        _check(lib.slh_write_constants(_b(self.constants), self.n, dptr(np.ascontiguousarray(group.R)),
                                       dptr(np.ascontiguousarray(group.m)), dptr(np.ascontiguousarray(group.moi)),
                                       precision), "constants")

    @property
    def simdata(self) -> str:
        return self.prefix + "simData.csv"

    @property
    def energy(self) -> str:
        return self.prefix + "energy.csv"

    @property
    def constants(self) -> str:
        return self.prefix + "constants.csv"

    def write_state(self, group: BallGroup) -> None:
        arr = [np.ascontiguousarray(a, dtype=np.float64) for a in (group.pos, group.w, group.vel)]
        _check(_lib.lib().slh_append_simdata_row(_b(self.simdata), self.n, *[dptr(a) for a in arr], self.precision),
               "simData row")

    def write_energy(self, row: EnergyRow, precision: int = ENERGY_PRECISION) -> None:
        _check(_lib.lib().slh_append_energy_row(_b(self.energy), row.time, row.PE, row.KE, row.p, row.L, precision),
               "energy row")


def load_continue(prefix: str | Path) -> BallGroup:
    """The last saved state of <prefix>simData.csv with <prefix>constants.csv."""
    lib = _lib.lib()
    prefix = str(prefix)
    n = ctypes.c_int(0)
    _check(lib.slh_count_last_state(_b(prefix + "simData.csv"), ctypes.byref(n)), "simData last line")
    g = BallGroup(n.value)
    pos, vel, w = (np.zeros(3 * n.value) for _ in range(3))
    _check(lib.slh_read_last_state(_b(prefix + "simData.csv"), n.value, dptr(pos), dptr(vel), dptr(w)),
           "simData parse")
    R, m, moi = (np.zeros(n.value) for _ in range(3))
    _check(lib.slh_read_constants(_b(prefix + "constants.csv"), n.value, dptr(R), dptr(m), dptr(moi)),
           "constants parse")
    g.pos[:] = pos.reshape(-1, 3); g.vel[:] = vel.reshape(-1, 3); g.w[:] = w.reshape(-1, 3)
    g.R[:] = R; g.m[:] = m; g.moi[:] = moi
    return g


def save_checkpoint(path: str | Path, group: BallGroup, pos_prev: np.ndarray, dt: float, kin: float, kout: float,
                    sim_time: float = 0.0, step: int = 0) -> None:
    arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in
            (group.pos, group.vel, group.w, group.acc, group.aacc, pos_prev, group.R, group.m, group.moi)]
    _check(_lib.lib().slh_write_checkpoint(_b(path), group.num_particles, *[dptr(a) for a in arrs], dt, kin, kout,
                                           sim_time, step), "checkpoint write")


def load_checkpoint(path: str | Path) -> dict:
    lib = _lib.lib()
    n = ctypes.c_int(0)
    dt, kin, kout, st = (ctypes.c_double() for _ in range(4))
    step = ctypes.c_longlong()
    _check(lib.slh_read_checkpoint_header(_b(path), ctypes.byref(n), ctypes.byref(dt), ctypes.byref(kin),
                                          ctypes.byref(kout), ctypes.byref(st), ctypes.byref(step)), "checkpoint")
    k = n.value
    v3 = [np.zeros(3 * k) for _ in range(6)]
    s1 = [np.zeros(k) for _ in range(3)]
    _check(lib.slh_read_checkpoint(_b(path), k, *[dptr(a) for a in v3 + s1]), "checkpoint read")
    g = BallGroup(k)
    g.pos[:], g.vel[:], g.w[:], g.acc[:], g.aacc[:] = (a.reshape(-1, 3) for a in v3[:5])
    g.R[:], g.m[:], g.moi[:] = s1
    return {"group": g, "pos_prev": v3[5].reshape(-1, 3), "dt": dt.value, "kin": kin.value, "kout": kout.value,
            "sim_time": st.value, "step": step.value}
