"""Collision-outcome surrogate: a 5-member ensemble of BF16 MLPs
(include/spacelab_mlp.h) trained on outcomes of collisions simulated by the
batched solver, used to screen a parameter sweep.

Features (8): N_t, N_p, log speed, normalised impact parameter, COR, mu, and
each cluster's radius of gyration (in sphere radii).  Outcomes (4): stuck
projectile mass fraction, largest-remnant mass fraction, final radius of
gyration of the largest remnant (in sphere radii), fraction of the initial
kinetic energy dissipated.  Inputs and outputs are standardised with the
training set's mean and standard deviation.
"""
from __future__ import annotations

import ctypes
import time

import numpy as np

from . import _lib
from ._lib import check

FEATURES = ("n_t", "n_p", "log_speed", "b_frac", "cor", "mu", "rg_t", "rg_p")
OUTCOMES = ("stuck_fraction", "largest_fraction", "rg_final", "dissipated_fraction")

_fp = ctypes.POINTER(ctypes.c_float)


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


class Mlp:
    """One network on the GPU."""

    def __init__(self, n_in: int, n_out: int, hidden: int = 256, layers: int = 4, max_batch: int = 1024,
                 seed: int = 0):
        self.lib = _lib.lib()
        self.n_in, self.n_out, self.hidden, self.layers = n_in, n_out, hidden, layers
        h = ctypes.c_void_p()
        check(self.lib.sl_mlp_create(n_in, hidden, layers, n_out, max_batch, seed, ctypes.byref(h)), "sl_mlp_create")
        self.h = h

    def close(self):
        if self.h:
            self.lib.sl_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def num_params(self) -> int:
        n = ctypes.c_int64()
        check(self.lib.sl_mlp_num_params(self.h, ctypes.byref(n)), "sl_mlp_num_params")
        return n.value

    def params(self) -> np.ndarray:
        p = np.zeros(self.num_params(), dtype=np.float32)
        check(self.lib.sl_mlp_get_params(self.h, p.ctypes.data_as(_fp)), "sl_mlp_get_params")
        return p

    def set_params(self, p: np.ndarray) -> None:
        p = _f32(p)
        check(self.lib.sl_mlp_set_params(self.h, p.ctypes.data_as(_fp)), "sl_mlp_set_params")

    def gradients(self, x: np.ndarray, y: np.ndarray) -> tuple[float, np.ndarray]:
        x, y = _f32(x), _f32(y)
        g = np.zeros(self.num_params(), dtype=np.float32)
        loss = ctypes.c_float()
        check(self.lib.sl_mlp_gradients(self.h, x.ctypes.data_as(_fp), y.ctypes.data_as(_fp), len(x),
                                        g.ctypes.data_as(_fp), ctypes.byref(loss)), "sl_mlp_gradients")
        return loss.value, g

    def train(self, x, y, epochs: int, batch: int = 256, lr: float = 1e-3, seed: int = 0) -> np.ndarray:
        x, y = _f32(x), _f32(y)
        curve = np.zeros(epochs, dtype=np.float32)
        check(self.lib.sl_mlp_train(self.h, x.ctypes.data_as(_fp), y.ctypes.data_as(_fp), len(x), epochs, batch, lr,
                                    seed, curve.ctypes.data_as(_fp)), "sl_mlp_train")
        return curve

    def predict(self, x) -> np.ndarray:
        x = _f32(x)
        y = np.zeros((len(x), self.n_out), dtype=np.float32)
        check(self.lib.sl_mlp_predict(self.h, x.ctypes.data_as(_fp), len(x), y.ctypes.data_as(_fp)), "sl_mlp_predict")
        return y


class Ensemble:
    """Five independently initialised networks on standardised data."""

    def __init__(self, n_in: int, n_out: int, members: int = 5, hidden: int = 256, layers: int = 4, seed: int = 0):
        self.nets = [Mlp(n_in, n_out, hidden, layers, seed=seed + 7919 * k) for k in range(members)]
        self.xm = self.xs = self.ym = self.ys = None

    def fit(self, x: np.ndarray, y: np.ndarray, epochs: int = 200, batch: int = 256, lr: float = 1e-3,
            seed: int = 0) -> dict:
        self.xm, self.xs = x.mean(0), x.std(0) + 1e-12
        self.ym, self.ys = y.mean(0), y.std(0) + 1e-12
        xn, yn = (x - self.xm) / self.xs, (y - self.ym) / self.ys
        t0 = time.perf_counter()
        curves = [net.train(xn, yn, epochs, batch, lr, seed + k) for k, net in enumerate(self.nets)]
        return {"seconds": time.perf_counter() - t0, "final_loss": [float(c[-1]) for c in curves],
                "curves": [c.tolist() for c in curves]}

    def predict(self, x: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
        """Ensemble mean and standard deviation in the outcomes' units."""
        xn = (x - self.xm) / self.xs
        preds = np.stack([net.predict(xn) * self.ys + self.ym for net in self.nets])
        return preds.mean(0), preds.std(0)

    def close(self):
        for n in self.nets:
            n.close()
