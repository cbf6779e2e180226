"""Collision sweeps: features and outcomes of simulated collisions, and the
surrogate-screened sweep.

Outcomes of one collision (after its last step):

- stuck fraction: the share of the projectile's mass that ends in the largest remnant;
- largest fraction: the largest remnant's share of the total mass;
- rg_final: the largest remnant's radius of gyration, in sphere radii;
- dissipated fraction: (E(0) - E(end)) / KE(0), from the energy records.

A remnant is a connected component of spheres whose surface gap is below h_min (see slh_collision_outcome).

Features are N_t, N_p, log speed, b/(R_t+R_p), COR, mu, and each cluster's
radius of gyration in sphere radii. The radius of gyration of a cluster packed
uniformly in a sphere is sqrt(3/5) R_c with R_c = a (N / phi)^(1/3); that
formula is used for every point, simulated or not.

``screen_sweep`` evaluates the ensemble on every sweep point. It then re-runs
with the plain FP64 method the points whose ensemble spread exceeds
``threshold`` on any standardised outcome, plus a random ``audit`` fraction,
and reports the surrogate error on the re-run points and the cost against
simulating every point.
"""
from __future__ import annotations

import ctypes
import time

import numpy as np

from . import _lib, configs
from . import batch as B
from ._lib import dptr

BOND_GAP = 0.1 * configs.RADIUS  # = h_min


def rg_formula(n) -> np.ndarray:
    return np.sqrt(3.0 / 5.0) * (np.asarray(n, dtype=np.float64) / configs.PHI) ** (1.0 / 3.0)


def features(cols: list[B.Collision]) -> np.ndarray:
    return np.array([[c.n_t, c.n_p, np.log(c.speed), c.b_frac, c.cor, c.mu, rg_formula(c.n_t), rg_formula(c.n_p)]
                     for c in cols], dtype=np.float64)


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


# Collision recipe of the surrogate study: the projectile's bounding sphere
# starts CLEARANCE sphere radii from the target's, and k comes from the
# reference formula at speed / K_SPEED_DIV (overlaps ~3% of a radius), so the
# STEPS-step window (contact time = 50 steps) covers the projectile
# travelling ~10 sphere radii into the target.
CLEARANCE = 0.2
K_SPEED_DIV = 30.0
STEPS = 4000
NT_RANGE = (64, 256)


def sample_params(count: int, seed: int, nt_range=NT_RANGE) -> list[B.Collision]:
    """Sweep points without building their clusters."""
    return B.sample_collisions(count, seed, nt_range=nt_range, build=False)


def build(c: B.Collision) -> B.Collision:
    return B.build_instance(c, CLEARANCE, K_SPEED_DIV)


def screen_sweep(ens, points: list[B.Collision], steps: int, threshold: float, audit: float, seed: int,
                 sim_mode: str = "exact", sim_cost_per_pair_eval: float | None = None,
                 max_uncertain: float | None = None) -> dict:
    """Screen a sweep with the ensemble, re-simulate uncertain + audit points
    with the FP64 method, and account the cost.  A point is uncertain when
    the ensemble's standard deviation on some outcome, in units of that
    outcome's training spread, exceeds `threshold`; with `max_uncertain` the
    threshold is raised to the spread quantile that flags at most that
    fraction of the sweep."""
    rng = np.random.default_rng(seed)
    X = features(points)
    t0 = time.perf_counter()
    mean, std = ens.predict(X)
    t_inf = time.perf_counter() - t0
    spread = (std / ens.ys).max(axis=1)
    if max_uncertain is not None:
        threshold = max(threshold, float(np.quantile(spread, 1.0 - max_uncertain)))
    uncertain = np.nonzero(spread > threshold)[0]
    audit_idx = rng.choice(len(points), size=max(1, int(round(audit * len(points)))), replace=False)
    rerun = np.union1d(uncertain, audit_idx)
    cols = [build(points[i]) for i in rerun]
    sim_out, info = simulate(cols, steps, sim_mode)
    err = np.abs(mean[rerun] - sim_out)
    aud_pos = np.searchsorted(rerun, np.sort(audit_idx))
    counts = np.array([p.n for p in points], dtype=np.float64)
    all_pair_evals = float((counts * (counts - 1) / 2).sum() * steps)
    rate = sim_cost_per_pair_eval or (info["seconds"] / info["pair_evals"])
    full_cost = all_pair_evals * rate
    screened_cost = t_inf + info["seconds"]
    return {"points": len(points), "uncertain": int(len(uncertain)), "audit": int(len(audit_idx)),
            "rerun": int(len(rerun)), "inference_s": t_inf, "rerun_sim_s": info["seconds"],
            "full_sim_s_estimate": full_cost, "cost_ratio": full_cost / screened_cost,
            "audit_mae": err[aud_pos].mean(0).tolist(), "audit_max_err": err[aud_pos].max(0).tolist(),
            "rerun_mae": err.mean(0).tolist(), "outcome_std": sim_out.std(0).tolist(),
            "threshold": threshold, "sim_mode": sim_mode}
