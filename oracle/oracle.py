"""ctypes wrappers of the CPU oracle (TEST INFRASTRUCTURE ONLY).

  CpuOracle  -- oracle/liboracle.so, the C restatement of the reference step
                (sl_oracle.c), built everywhere by spacelab_gb300.build.
  RefPin     -- oracle/_ref/libslref.so, the reference's own sim_one_step
                compiled from the reference sources (ref_harness.cpp,
                -O2 -ffp-contract=off), or oracle/_ref/libslref_native.so,
                the same TU at -O3 -march=native (timing only); only where
                the reference tree or its snapshot was at hand at build time.

Only the tests, __graft_entry__.smoke() and bench.py's CPU-baseline legs use
this module, as the checker; the GPU library never does.
"""
from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ORACLE_LIB = HERE / "liboracle.so"
REF_LIB = HERE / "_ref" / "libslref.so"
REF_LIB_NATIVE = HERE / "_ref" / "libslref_native.so"
REF_LIB_GPU = HERE / "_ref" / "libslref_gpu.so"  # the reference TU with the GPU adapter (make adapter)
_P = ctypes.POINTER(ctypes.c_double)


def _p(a):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_P)


class _Mat(ctypes.Structure):
    _fields_ = [(k, ctypes.c_double) for k in ("G", "Ha", "u_s", "u_r", "h_min")]


_olib = None


def _oracle_lib():
    global _olib
    if _olib is None:
        if not ORACLE_LIB.exists():
            raise ImportError(f"{ORACLE_LIB} missing: run `python -m spacelab_gb300.build`")
        lib = ctypes.CDLL(str(ORACLE_LIB))
        lib.slo_create.restype = ctypes.c_void_p
        lib.slo_create.argtypes = [ctypes.c_int, _P, _P, _P, ctypes.POINTER(_Mat)]
        lib.slo_destroy.argtypes = [ctypes.c_void_p]
        lib.slo_set_state.argtypes = [ctypes.c_void_p, _P, _P, _P]
        lib.slo_set_acc.argtypes = [ctypes.c_void_p, _P, _P]
        lib.slo_set_scalars.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_double, ctypes.c_double]
        lib.slo_set_prev_positions.argtypes = [ctypes.c_void_p, _P]
        lib.slo_init.argtypes = [ctypes.c_void_p, _P]
        lib.slo_step.argtypes = [ctypes.c_void_p, ctypes.c_int, _P]
        lib.slo_step_rows.argtypes = [ctypes.c_void_p, ctypes.c_int, _P, ctypes.c_int]
        lib.slo_get_state.argtypes = [ctypes.c_void_p, _P, _P, _P, _P, _P]
        lib.slo_contacts.restype = ctypes.c_long
        lib.slo_contacts.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int), ctypes.c_long]
        lib.slo_max_threads.restype = ctypes.c_int
        for f in ("slo_destroy", "slo_set_state", "slo_set_acc", "slo_set_scalars", "slo_set_prev_positions",
                  "slo_init", "slo_step", "slo_step_rows", "slo_get_state"):
            getattr(lib, f).restype = None
        _olib = lib
    return _olib


def material_tuple(mat) -> tuple:
    return (mat.G, mat.Ha, mat.u_s, mat.u_r, mat.h_min)


class CpuOracle:
    """The C restatement of sim_one_step on one system (double, AoS)."""

    def __init__(self, pos, vel, w, R, m, moi, material, dt, kin, kout):
        lib = _oracle_lib()
        self.lib = lib
        self.n = len(R)
        R, m, moi = (np.ascontiguousarray(x, dtype=np.float64) for x in (R, m, moi))
        self._mat = _Mat(*material_tuple(material))
        self.h = lib.slo_create(self.n, _p(R), _p(m), _p(moi), ctypes.byref(self._mat))
        if not self.h:
            raise MemoryError("slo_create failed")
        self.set_state(pos, vel, w)
        lib.slo_set_scalars(self.h, dt, kin, kout)

    def set_state(self, pos, vel, w):
        arrs = [np.ascontiguousarray(np.asarray(x, dtype=np.float64).reshape(-1)) for x in (pos, vel, w)]
        self.lib.slo_set_state(self.h, *[_p(a) for a in arrs])

    def set_scalars(self, dt, kin, kout):
        self.lib.slo_set_scalars(self.h, dt, kin, kout)

    def init(self) -> np.ndarray:
        e = np.zeros(8)
        self.lib.slo_init(self.h, _p(e))
        return e

    def step(self, write: bool = False, threads: int | None = None) -> np.ndarray:
        """One step; threads=None runs the sequential reference loop order,
        an int runs the row-parallel variant (bit-identical state)."""
        e = np.zeros(8)
        if threads is None:
            self.lib.slo_step(self.h, int(write), _p(e))
        else:
            self.lib.slo_step_rows(self.h, int(write), _p(e), int(threads))
        return e

    def state(self) -> dict:
        out = {k: np.zeros(3 * self.n) for k in ("pos", "vel", "w", "acc", "aacc")}
        self.lib.slo_get_state(self.h, *[_p(out[k]) for k in ("pos", "vel", "w", "acc", "aacc")])
        return {k: v.reshape(-1, 3) for k, v in out.items()}

    def contacts(self) -> np.ndarray:
        cnt = self.lib.slo_contacts(self.h, None, 0)
        buf = np.zeros(2 * max(1, cnt), dtype=np.int32)
        self.lib.slo_contacts(self.h, buf.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), cnt)
        return buf[: 2 * cnt].reshape(-1, 2)

    def close(self):
        if self.h:
            self.lib.slo_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def max_threads() -> int:
        return int(_oracle_lib().slo_max_threads())


_rlibs: dict = {}


def ref_available(native: bool = False) -> bool:
    return (REF_LIB_NATIVE if native else REF_LIB).exists()


def _ref_lib(native: bool, path: Path | None = None):
    path = path or (REF_LIB_NATIVE if native else REF_LIB)
    if path not in _rlibs:
        # RTLD_LOCAL (ctypes' default): each build keeps its own globals
        lib = ctypes.CDLL(str(path))
        lib.slref_material.argtypes = [_P]
        lib.slref_material.restype = None
        lib.slref_init.argtypes = [ctypes.c_int, _P, _P, _P, _P, _P, _P, ctypes.c_double, ctypes.c_double,
                                   ctypes.c_double, _P]
        lib.slref_init.restype = ctypes.c_int
        lib.slref_step.argtypes = [ctypes.c_int, _P]
        lib.slref_step.restype = None
        lib.slref_get.argtypes = [_P] * 5
        lib.slref_get.restype = None
        lib.slref_resume.argtypes = [_P] * 6
        lib.slref_resume.restype = ctypes.c_int
        lib.slref_looper.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, _P]
        lib.slref_looper.restype = ctypes.c_char_p
        _rlibs[path] = lib
    return _rlibs[path]


class RefPin:
    """The reference's own sim_one_step (one global system per process and
    build).  native=True selects the -O3 -march=native build, whose results
    may differ in the last bits (contracted multiply-adds)."""

    def __init__(self, pos, vel, w, R, m, moi, dt, kin, kout, native: bool = False, lib_path: Path | None = None):
        self.lib = _ref_lib(native, lib_path)
        self.n = len(R)
        arrs = [np.ascontiguousarray(np.asarray(x, dtype=np.float64).reshape(-1)) for x in (pos, vel, w, R, m, moi)]
        self.e0 = np.zeros(8)
        rc = self.lib.slref_init(self.n, *[_p(a) for a in arrs], dt, kin, kout, _p(self.e0))
        if rc != 0:
            raise RuntimeError("slref_init failed")

    def resume(self, pos, vel, w, acc, aacc, pos_prev=None):
        """Continue from a saved state: acc/aacc of its last force pass and
        the positions of the step before it (NULL = pos)."""
        arrs = [np.ascontiguousarray(np.asarray(x, dtype=np.float64).reshape(-1)) for x in (pos, vel, w, acc, aacc)]
        prev = None if pos_prev is None else np.ascontiguousarray(np.asarray(pos_prev, dtype=np.float64).reshape(-1))
        if self.lib.slref_resume(*[_p(a) for a in arrs], _p(prev)) != 0:
            raise RuntimeError("slref_resume failed")

    def looper(self, prefix: str, steps: int, skip: int) -> str:
        """The reference's sim_init_write + sim_looper into files named
        <prefix>simData.csv, <prefix>energy.csv, <prefix>constants.csv;
        returns the prefix the writer used."""
        return self.lib.slref_looper(prefix.encode(), int(steps), int(skip), _p(self.e0)).decode()

    @staticmethod
    def material() -> tuple:
        if not REF_LIB.exists():
            raise ImportError("reference pin not built")
        lib = ctypes.CDLL(str(REF_LIB))
        out = np.zeros(5)
        lib.slref_material.argtypes = [_P]
        lib.slref_material(_p(out))
        return tuple(out)

    def step(self, write: bool = False) -> np.ndarray:
        e = np.zeros(8)
        self.lib.slref_step(int(write), _p(e))
        return e

    def state(self) -> dict:
        out = {k: np.zeros(3 * self.n) for k in ("pos", "vel", "w", "acc", "aacc")}
        self.lib.slref_get(*[_p(out[k]) for k in ("pos", "vel", "w", "acc", "aacc")])
        return {k: v.reshape(-1, 3) for k, v in out.items()}
