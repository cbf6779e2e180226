"""ctypes binding of libspacelab_gb300.so (include/spacelab_gpu.h and
include/spacelab_host.h).

The library is the product: there is no Python or CPU fallback.  If it is
missing, importing this module raises, naming the build command.
"""
from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "libspacelab_gb300.so"

SL_OK = 0
SL_ERR_ARG = 1
SL_ERR_CUDA = 2
SL_ERR_NONFINITE = 3
SL_ERR_ALLOC = 4
SL_ERR_STATE = 5
SL_ERR_UNSUPPORTED = 6
SL_ERR_TIMEOUT = 7

SL_MODE_EXACT = 0
SL_MODE_MIXED = 1
API_VERSION = 2  # SL_API_VERSION of include/spacelab_gpu.h
SL_MODE_MIXED_DF = 2

_c_double_p = ctypes.POINTER(ctypes.c_double)
_c_int_p = ctypes.POINTER(ctypes.c_int)


class Material(ctypes.Structure):
    """sl_material: G, Ha, u_s, u_r, h_min (dust_const.hpp:21-38)."""

    _fields_ = [("G", ctypes.c_double), ("Ha", ctypes.c_double), ("u_s", ctypes.c_double),
                ("u_r", ctypes.c_double), ("h_min", ctypes.c_double)]


class Energy(ctypes.Structure):
    """sl_energy: the totals of one write step."""

    _fields_ = [("PE", ctypes.c_double), ("KE", ctypes.c_double), ("mom", ctypes.c_double * 3),
                ("ang_mom", ctypes.c_double * 3)]

    def as_array(self) -> np.ndarray:
        return np.array([self.PE, self.KE, *self.mom, *self.ang_mom], dtype=np.float64)


class SpaceLabError(RuntimeError):
    def __init__(self, code: int, where: str, msg: str):
        super().__init__(f"{where} failed with status {code}: {msg}")
        self.code = code


# (name, restype, argtypes)
_PROTOS = [
    ("sl_version", ctypes.c_int, []),
    ("sl_last_error", ctypes.c_char_p, []),
    ("sl_create", ctypes.c_int, [ctypes.c_int, ctypes.POINTER(Material), ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]),
    ("sl_destroy", ctypes.c_int, [ctypes.c_void_p]),
    ("sl_num_particles", ctypes.c_int, [ctypes.c_void_p, _c_int_p]),
    ("sl_upload", ctypes.c_int, [ctypes.c_void_p] + [_c_double_p] * 6),
    ("sl_upload_resume", ctypes.c_int, [ctypes.c_void_p] + [_c_double_p] * 6),
    ("sl_set_scalars", ctypes.c_int, [ctypes.c_void_p, ctypes.c_double, ctypes.c_double, ctypes.c_double]),
    ("sl_init_forces", ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Energy)]),
    ("sl_step", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.POINTER(Energy)]),
    ("sl_run", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.POINTER(Energy),
                              ctypes.c_int, _c_int_p]),
    ("sl_download", ctypes.c_int, [ctypes.c_void_p] + [_c_double_p] * 5),
    ("sl_step_host", ctypes.c_int, [ctypes.c_void_p] + [_c_double_p] * 5 + [ctypes.c_int, ctypes.POINTER(Energy)]),
    ("sl_contacts", ctypes.c_int, [ctypes.c_void_p, _c_int_p, ctypes.c_long, ctypes.POINTER(ctypes.c_long)]),
    ("sl_stream", ctypes.c_void_p, [ctypes.c_void_p]),
    ("sl_set_overlap", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    ("sl_set_rowsum", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    ("sl_step_launches", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]),
    ("sl_pair_kernel", ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_char_p)]),
    ("sl_kernel_timing", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    ("sl_kernel_times", ctypes.c_int, [ctypes.c_void_p, _c_double_p, _c_double_p, ctypes.POINTER(ctypes.c_long),
                                       ctypes.c_int]),
    ("sl_device_bytes", ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint64)]),
    ("sl_forces_static", ctypes.c_int, [ctypes.c_int] + [ctypes.c_void_p] * 6 + [ctypes.POINTER(Material),
                                        ctypes.c_double, ctypes.c_double] + [ctypes.c_void_p] * 4),
    # batched solver (spacelab_batch.h)
    ("sl_batch_create", ctypes.c_int, [ctypes.c_int, _c_int_p, ctypes.POINTER(Material), ctypes.c_int, ctypes.c_int,
                                       ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]),
    ("sl_batch_destroy", ctypes.c_int, [ctypes.c_void_p]),
    ("sl_batch_upload", ctypes.c_int, [ctypes.c_void_p] + [_c_double_p] * 10),
    ("sl_batch_set_shape", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]),
    ("sl_batch_shape", ctypes.c_int, [ctypes.c_void_p, _c_int_p, _c_int_p, _c_int_p]),
    ("sl_batch_autotune", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, _c_int_p, _c_int_p, _c_double_p]),
    ("sl_batch_run", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    ("sl_batch_download", ctypes.c_int, [ctypes.c_void_p] + [_c_double_p] * 5),
    ("sl_batch_energy", ctypes.c_int, [ctypes.c_void_p, _c_double_p, _c_int_p]),
    ("sl_batch_status", ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint)]),
    # surrogate network (spacelab_mlp.h)
    ("sl_mlp_create", ctypes.c_int, [ctypes.c_int] * 5 + [ctypes.c_uint64, ctypes.POINTER(ctypes.c_void_p)]),
    ("sl_mlp_destroy", ctypes.c_int, [ctypes.c_void_p]),
    ("sl_mlp_num_params", ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64)]),
    ("sl_mlp_get_params", ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_float)]),
    ("sl_mlp_set_params", ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_float)]),
    ("sl_mlp_gradients", ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float),
                                        ctypes.c_int, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float)]),
    ("sl_mlp_train", ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float),
                                    ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_float, ctypes.c_uint64,
                                    ctypes.POINTER(ctypes.c_float)]),
    ("sl_mlp_predict", ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_float), ctypes.c_int,
                                      ctypes.POINTER(ctypes.c_float)]),
    # diagnostics (spacelab_diag.h)
    ("sl_diag_division", ctypes.c_int, [ctypes.c_int] + [_c_double_p] * 4),
    ("sl_diag_fp64_peak", ctypes.c_int, [_c_double_p]),
    ("sl_diag_fp32_peak", ctypes.c_int, [_c_double_p]),
    ("sl_diag_gemm_bf16", ctypes.c_int, [ctypes.c_int] * 3 + [ctypes.POINTER(ctypes.c_uint16)] * 2 +
     [ctypes.POINTER(ctypes.c_float), ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_float),
      ctypes.POINTER(ctypes.c_uint16)]),
    ("sl_diag_fp64_add_latency", ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_double)]),
    ("sl_diag_exact_ops", ctypes.c_int, [ctypes.c_int] + [_c_double_p] * 3),
    ("sl_diag_int_ops", ctypes.c_int, [ctypes.c_int] + [_c_double_p] * 3),
    # host setup (spacelab_host.h)
    ("slh_build_cluster", ctypes.c_int, [ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                         ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                         ctypes.c_uint64] + [_c_double_p] * 6),
    ("slh_build_collision", ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                           ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                           ctypes.c_double, ctypes.c_uint64, ctypes.c_uint64] + [_c_double_p] * 6),
    ("slh_spring_and_dt", ctypes.c_int, [ctypes.c_double] * 6 + [_c_double_p] * 3),
    ("slh_to_origin", ctypes.c_int, [ctypes.c_int, _c_double_p, _c_double_p]),
    ("slh_cluster_rg", ctypes.c_int, [ctypes.c_int, _c_int_p, ctypes.POINTER(ctypes.c_uint64), ctypes.c_double,
                                      ctypes.c_double, ctypes.c_double, ctypes.c_int, _c_double_p]),
    ("slh_write_simdata_header", ctypes.c_int, [ctypes.c_char_p, ctypes.c_int]),
    ("slh_append_simdata_row", ctypes.c_int, [ctypes.c_char_p, ctypes.c_int] + [_c_double_p] * 3 + [ctypes.c_int]),
    ("slh_write_energy_header", ctypes.c_int, [ctypes.c_char_p]),
    ("slh_append_energy_row", ctypes.c_int, [ctypes.c_char_p] + [ctypes.c_double] * 5 + [ctypes.c_int]),
    ("slh_write_constants", ctypes.c_int, [ctypes.c_char_p, ctypes.c_int] + [_c_double_p] * 3 + [ctypes.c_int]),
    ("slh_count_last_state", ctypes.c_int, [ctypes.c_char_p, _c_int_p]),
    ("slh_read_last_state", ctypes.c_int, [ctypes.c_char_p, ctypes.c_int] + [_c_double_p] * 3),
    ("slh_read_constants", ctypes.c_int, [ctypes.c_char_p, ctypes.c_int] + [_c_double_p] * 3),
    ("slh_write_checkpoint", ctypes.c_int, [ctypes.c_char_p, ctypes.c_int] + [_c_double_p] * 9 +
     [ctypes.c_double] * 4 + [ctypes.c_longlong]),
    ("slh_read_checkpoint_header", ctypes.c_int, [ctypes.c_char_p, _c_int_p] + [_c_double_p] * 4 +
     [ctypes.POINTER(ctypes.c_longlong)]),
    ("slh_read_checkpoint", ctypes.c_int, [ctypes.c_char_p, ctypes.c_int] + [_c_double_p] * 9),
    ("slh_collision_outcome", ctypes.c_int, [ctypes.c_int, ctypes.c_int] + [_c_double_p] * 3 + [ctypes.c_double] +
     [_c_double_p] * 3 + [_c_int_p]),
    ("slh_radius_of_gyration", ctypes.c_int, [ctypes.c_int, _c_double_p, _c_double_p, _c_double_p]),
    ("slh_log", ctypes.c_double, [ctypes.c_double]),
    ("slh_exp", ctypes.c_double, [ctypes.c_double]),
    ("slh_rng_next", ctypes.c_uint64, [ctypes.POINTER(ctypes.c_uint64)]),
]

EXPORTED_SYMBOLS = [name for name, _, _ in _PROTOS]


def load(path: Path | str = LIB_PATH) -> ctypes.CDLL:
    path = Path(path)
    if not path.exists():
        raise ImportError(
            f"{path} is missing: build it with `python -m spacelab_gb300.build` "
            "(the GPU step has no CPU fallback)")
    lib = ctypes.CDLL(str(path))
    for name, res, args in _PROTOS:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if lib.sl_version() != API_VERSION:
        raise ImportError(f"{path}: ABI version {lib.sl_version()} != {API_VERSION}")
    return lib


_LIB: ctypes.CDLL | None = None


def lib() -> ctypes.CDLL:
    global _LIB
    if _LIB is None:
        _LIB = load()
    return _LIB


def check(code: int, where: str) -> None:
    if code != SL_OK:
        msg = lib().sl_last_error()
        raise SpaceLabError(code, where, msg.decode() if msg else "")


def dptr(a: np.ndarray):
    """Pointer to a C-contiguous float64 array (None passes NULL)."""
    if a is None:
        return None
    if a.dtype != np.float64 or not a.flags["C_CONTIGUOUS"]:
        raise TypeError("expected a C-contiguous float64 array")
    return a.ctypes.data_as(_c_double_p)
