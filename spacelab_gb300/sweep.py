"""Collision sweeps: features and outcomes of simulated collisions, and the
surrogate-screened sweep.

Outcomes of one collision (after its last step):

- stuck fraction: the share of the projectile's mass that ends in the largest remnant;
- largest fraction: the largest remnant's share of the total mass;
- rg_final: the largest remnant's radius of gyration, in sphere radii;
- dissipated fraction: (E(0) - E(end)) / KE(0), from the energy records.

A remnant is a connected component of spheres whose surface gap is below h_min (see slh_collision_outcome).

Features are N_t, N_p, log speed, b/(R_t+R_p), COR, mu, and each cluster's
measured radius of gyration in sphere radii: the clusters a point's seeds
build (slh_cluster_rg builds them on all host threads and keeps only Rg),
simulated or not.

The collisions are the batched solver's sweep (batch.sample_collisions):
N_t uniform in [64, 1600], centres 1.1 (R_t + R_p) apart, k at 1/50 of the
impact speed, STEPS = 3000 steps.

``pick_threshold`` chooses the ensemble-spread threshold on held-out
validation collisions: the largest threshold at which the accepted
validation points' mean absolute error stays within a stated fraction of
each outcome's spread.  ``screen_sweep`` evaluates the ensemble on every
sweep point, re-runs with the simulator the points whose spread exceeds the
threshold plus a random ``audit`` fraction, and reports the surrogate error
on the re-run points and the cost against simulating every point.
"""
from __future__ import annotations

import ctypes
import time

import numpy as np

from . import _lib, configs
from . import batch as B
from ._lib import dptr

BOND_GAP = 0.1 * configs.RADIUS  # = h_min


def cluster_rg(n: np.ndarray, seeds: np.ndarray, threads: int = 0) -> np.ndarray:
    """Radius of gyration, in sphere radii, of the monodisperse cluster that
    each (n, seed) builds (include/spacelab_host.h slh_cluster_rg)."""
    n = np.ascontiguousarray(n, dtype=np.int32)
    seeds = np.ascontiguousarray(seeds, dtype=np.uint64)
    rg = np.zeros(len(n))
    rc = _lib.lib().slh_cluster_rg(len(n), n.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                   seeds.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), configs.RADIUS,
                                   configs.DENSITY, configs.PHI, threads, dptr(rg))
    if rc != 0:
        raise RuntimeError(f"slh_cluster_rg failed ({rc})")
    return rg / configs.RADIUS


def features(cols: list[B.Collision]) -> np.ndarray:
    seeds = np.array([B.cluster_seeds(c) for c in cols], dtype=np.uint64).reshape(-1, 2)
    nt = np.array([c.n_t for c in cols])
    npj = np.array([c.n_p for c in cols])
    rg = cluster_rg(np.concatenate([nt, npj]), np.concatenate([seeds[:, 0], seeds[:, 1]]))
    rg_t, rg_p = rg[: len(cols)], rg[len(cols):]
    return np.array([[c.n_t, c.n_p, np.log(c.speed), c.b_frac, c.cor, c.mu, a, b]
                     for c, a, b in zip(cols, rg_t, rg_p)], dtype=np.float64)


def outcome(c: B.Collision, pos: np.ndarray, e_first: np.ndarray, e_last: np.ndarray) -> np.ndarray:
    lib = _lib.lib()
    lf, sf, rg = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    nc = ctypes.c_int()
    p = np.ascontiguousarray(pos.reshape(-1))
    rc = lib.slh_collision_outcome(c.n, c.n_t, dptr(p), dptr(np.ascontiguousarray(c.group.R)),
                                   dptr(np.ascontiguousarray(c.group.m)), BOND_GAP, ctypes.byref(lf),
                                   ctypes.byref(sf), ctypes.byref(rg), ctypes.byref(nc))
    if rc != 0:
        raise RuntimeError("slh_collision_outcome failed")
    E0 = e_first[0] + e_first[1]
    E1 = e_last[0] + e_last[1]
    diss = (E0 - E1) / e_first[1] if e_first[1] > 0 else 0.0
    return np.array([sf.value, lf.value, rg.value / configs.RADIUS, diss])


def simulate(cols: list[B.Collision], steps: int, mode: str = "mixed_df", skip: int | None = None,
             autotune: bool = True) -> tuple[np.ndarray, dict]:
    """Run the collisions through the batched solver; returns (outcomes, info)."""
    skip = steps if skip is None else skip
    run = B.BatchRun(cols, mode, steps=steps, skip=skip)
    tuned = run.autotune(sample_steps=2) if autotune else None
    wall = run.run(1, steps, do_init=True)
    st = run.state()
    en = run.energy()
    bad = run.status()
    out = np.array([outcome(c, run.instance_state(st, i)["pos"], en[i][0], en[i][-1]) for i, c in enumerate(cols)])
    counts = np.array([c.n for c in cols], dtype=np.float64)
    info = {"seconds": wall, "collisions": len(cols), "steps": steps, "mode": mode, "autotune": tuned,
            "pair_evals": float((counts * (counts - 1) / 2).sum() * steps), "nonfinite": int(bad.sum())}
    run.close()
    return out, info


# Collision recipe of the surrogate study: the batched solver's sweep of
# collisions (batch.sample_collisions), simulated for STEPS steps.
CLEARANCE = None     # centres 1.1 (R_t + R_p) apart
K_SPEED_DIV = 50.0   # k at 1/50 of the impact speed
STEPS = 3000
NT_RANGE = (64, 1600)


def sample_params(count: int, seed: int, nt_range=NT_RANGE) -> list[B.Collision]:
    """Sweep points without building their clusters."""
    return B.sample_collisions(count, seed, nt_range=nt_range, build=False)


def build(c: B.Collision) -> B.Collision:
    return B.build_instance(c, CLEARANCE, K_SPEED_DIV)


def pick_threshold(ens, x_val: np.ndarray, y_val: np.ndarray, error_target: float, min_accept: int = 20) -> dict:
    """The largest ensemble-spread threshold at which the validation points
    it accepts (spread <= threshold) have a mean absolute error of at most
    error_target x that outcome's training spread, on every outcome.  The
    spread of a point is max over outcomes of (ensemble std / outcome
    spread).  Returns the threshold, the accepted fraction of the validation
    set and the accepted points' standardised mean absolute errors."""
    mean, std = ens.predict(x_val)
    spread = (std / ens.ys).max(axis=1)
    err = np.abs(mean - y_val) / ens.ys
    order = np.argsort(spread)
    cum = np.cumsum(err[order], axis=0) / np.arange(1, len(order) + 1)[:, None]
    ok = np.all(cum <= error_target, axis=1)
    ok[: min_accept - 1] = False
    if not ok.any():
        return {"threshold": 0.0, "accept_fraction": 0.0, "mae_std_units": None, "error_target": error_target}
    k = int(np.nonzero(ok)[0].max())
    thr = float(spread[order[k]])
    acc = spread <= thr
    return {"threshold": thr, "accept_fraction": float(acc.mean()), "error_target": error_target,
            "mae_std_units": err[acc].mean(0).tolist(),
            "mae_std_units_all": err.mean(0).tolist()}


def screen_sweep(ens, points: list[B.Collision], steps: int, threshold: float, audit: float, seed: int,
                 sim_mode: str = "mixed_df", fp64_check: int = 0) -> dict:
    """Screen a sweep with the ensemble, re-simulate uncertain + audit points
    (sim_mode), and account the cost.  A point is uncertain when the
    ensemble's standard deviation on some outcome, in units of that
    outcome's training spread, exceeds `threshold`.  fp64_check > 0 re-runs
    that many audit points with the FP64 exact method too and reports how
    far its outcomes are from sim_mode's."""
    rng = np.random.default_rng(seed)
    t0 = time.perf_counter()
    X = features(points)
    t_feat = time.perf_counter() - t0
    t0 = time.perf_counter()
    mean, std = ens.predict(X)
    t_inf = time.perf_counter() - t0
    spread = (std / ens.ys).max(axis=1)
    uncertain = np.nonzero(spread > threshold)[0]
    audit_idx = rng.choice(len(points), size=max(1, int(round(audit * len(points)))), replace=False)
    rerun = np.union1d(uncertain, audit_idx)
    cols = [build(points[i]) for i in rerun]
    sim_out, info = simulate(cols, steps, sim_mode)
    err = np.abs(mean[rerun] - sim_out)
    aud_pos = np.searchsorted(rerun, np.sort(audit_idx))
    counts = np.array([p.n for p in points], dtype=np.float64)
    all_pair_evals = float((counts * (counts - 1) / 2).sum() * steps)
    rate = info["seconds"] / info["pair_evals"]
    full_cost = all_pair_evals * rate
    screened_cost = t_feat + t_inf + info["seconds"]
    out = {"points": len(points), "uncertain": int(len(uncertain)), "audit": int(len(audit_idx)),
           "rerun": int(len(rerun)), "rerun_fraction": len(rerun) / len(points),
           "uncertain_fraction": len(uncertain) / len(points),
           "features_s": t_feat, "inference_s": t_inf, "rerun_sim_s": info["seconds"],
           "full_sim_s_estimate": full_cost, "cost_ratio": full_cost / screened_cost,
           "audit_mae": err[aud_pos].mean(0).tolist(), "audit_max_err": err[aud_pos].max(0).tolist(),
           # the method without the network: the training mean for every point
           "audit_mae_training_mean": np.abs(ens.ym - sim_out[aud_pos]).mean(0).tolist(),
           "audit_mae_std_units": (err[aud_pos].mean(0) / ens.ys).tolist(),
           "rerun_mae": err.mean(0).tolist(), "outcome_std": sim_out.std(0).tolist(),
           "threshold": threshold, "sim_mode": sim_mode, "rerun_nonfinite": info["nonfinite"]}
    if fp64_check > 0:
        pick = np.sort(audit_idx)[:fp64_check]
        ex_out, ex_info = simulate([cols[int(np.searchsorted(rerun, i))] for i in pick], steps, "exact")
        diff = np.abs(ex_out - sim_out[np.searchsorted(rerun, pick)])
        out["fp64_check"] = {"collisions": len(pick), "mean_abs_diff": diff.mean(0).tolist(),
                             "max_abs_diff": diff.max(0).tolist(), "seconds": ex_info["seconds"],
                             "surrogate_mae_vs_fp64": np.abs(mean[pick] - ex_out).mean(0).tolist()}
    return out
