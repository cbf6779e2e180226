"""Benchmark of SpaceLab's step on GB300: pair-interactions/s at N=5000.

Workload: the aggregate collision of a 4000-sphere target and a 1000-sphere
projectile (seeded synthetic clusters; no dataset is involved), FP64, the
reference's write schedule (energy every 100 steps).  One bench step is one
velocity-Verlet step (sim_one_step); a pair interaction is one unordered
pair evaluated per step, N(N-1)/2 per step.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0).  `value` is device-resident throughput (state
in HBM, CUDA events on the library's stream); `e2e` is the same metric
through the C ABI from pinned host buffers, with the state uploaded and
downloaded every step; `roofline` reports the pair kernel against the FP64
pipe; `cpu_baseline` times the CPU oracle (a restatement of the reference
step, bit-identical to it) on a bounded sample on this host's cores.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "pair-interactions/s at N=5000 (FP64 aggregate collision)"
UNIT = "pair-interactions/s"


def _dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(
        os.environ.get("LOCAL_RANK", "0"))


def _workload():
    from spacelab_gb300 import configs
    return configs.aggregate_collision_5000()


def _config(w, extra=None):
    cfg = {"workload": w.name, "n_spheres": w.n, "n_target": 4000, "n_projectile": 1000, "steps_per_write": w.skip,
           "dt_s": w.dt, "kin": w.kin, "kout": w.kout, "seeds": w.info,
           "l2": "per-step working set > L2: the pair-term buffer (3*npad^2 doubles, 606 MB) is streamed "
                 "through HBM every step"}
    if extra:
        cfg.update(extra)
    return cfg


# ------------------------------------------------------------------ clocks --
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.proc = None
        self.path = ROOT / "gpurun_out" / f"clocks_rank{gpu_index}.csv"
        self.gpu = gpu_index

    def start(self):
        try:
            self.path.parent.mkdir(exist_ok=True)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.fh,
                                         stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.fh.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.path.read_text().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(smax)), "reasons": sorted(reasons),
                "samples": len(sm)}


# ------------------------------------------------------------- CPU oracle --
def cpu_oracle_rate(w, budget_s: float, threads: int = 0) -> dict:
    """Row-parallel CPU oracle on `threads` host threads (0 = all); steps of
    the same workload until budget_s elapses (at least 2)."""
    from oracle.oracle import CpuOracle
    g = w.group
    o = CpuOracle(g.pos, g.vel, g.w, g.R, g.m, g.moi, w.material, w.dt, w.kin, w.kout)
    o.init()
    o.step(False, threads=threads)  # warm-up
    t0 = time.perf_counter()
    steps = 0
    while True:
        o.step(False, threads=threads)
        steps += 1
        el = time.perf_counter() - t0
        if steps >= 2 and el >= budget_s:
            break
    cores = CpuOracle.max_threads() if threads == 0 else threads
    return {"value": w.pairs_per_step * steps / el, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"{steps} steps of the N=5000 workload ({el:.1f} s), row-parallel C restatement of "
                      f"sim_one_step (bit-identical to the reference build), {cores} threads, "
                      f"{os.uname().machine} host"}


def ref_pin_rate(w, budget_s: float) -> dict:
    """The reference's own sim_one_step (oracle/_ref, built from the reference
    sources where they are present), one thread, bounded sample."""
    from oracle.oracle import RefPin
    g = w.group
    ref = RefPin(g.pos, g.vel, g.w, g.R, g.m, g.moi, w.dt, w.kin, w.kout)
    ref.step(False)
    t0 = time.perf_counter()
    steps = 0
    while True:
        ref.step(False)
        steps += 1
        el = time.perf_counter() - t0
        if steps >= 2 and el >= budget_s:
            break
    return {"value": w.pairs_per_step * steps / el, "unit": UNIT, "cores": 1, "kind": "reference",
            "sample": f"{steps} steps of the N=5000 workload ({el:.1f} s), the reference's sim_one_step "
                      f"compiled from its sources (-O2 -ffp-contract=off), 1 thread"}


# ------------------------------------------------------------------ ours --
def run_ours(args, rank, world, local_rank) -> dict | None:
    import torch
    torch.cuda.set_device(local_rank)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from spacelab_gb300 import GpuStep, _lib
    from spacelab_gb300 import flops as F

    w = _workload()
    g = w.group
    sim = GpuStep(g.copy(), w.material, "exact")
    sim.set_scalars(w.dt, w.kin, w.kout)
    sim.init_conditions()
    stream = torch.cuda.ExternalStream(sim.stream_ptr())

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
            torch.cuda.synchronize()

    # warm-up (writes included so both pair-kernel variants are loaded)
    sim.sim_looper(steps=1 + args.warmup, skip=w.skip)
    first = 1 + args.warmup
    nwrites = sum(1 for s in range(first, first + args.steps) if s % w.skip == 0)

    clocks = ClockSampler(local_rank)
    barrier()
    clocks.start()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    sim.sim_looper(steps=first + args.steps, skip=w.skip, first_step=first)
    ev1.record(stream)
    barrier()
    clk = clocks.stop()
    ms = ev0.elapsed_time(ev1)
    t = torch.tensor([ms], dtype=torch.float64, device="cuda")
    if world > 1:
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    ms_max = float(t.item())
    pairs = w.pairs_per_step * args.steps * world
    value = pairs / (ms_max * 1e-3)
    gpu_launches = 3 * args.steps + 2 * nwrites

    # per-kernel timing of the pair kernel (non-write steps), same stream
    sim.kernel_timing(True)
    nk = max(10, min(50, args.steps))
    sim.step(nk, write_last=False)
    pair_ms, rowsum_ms, launches = sim.kernel_times(reset=True)
    sim.kernel_timing(False)
    contacts = int(len(sim.contacts()))
    pair_ms_avg = pair_ms / launches
    flops_launch = F.pair_flops(w.pairs_per_step, contacts, write=False)
    peak = _lib.lib()
    pk = __import__("ctypes").c_double()
    _lib.check(peak.sl_diag_fp64_peak(__import__("ctypes").byref(pk)), "sl_diag_fp64_peak")
    peak_tflops = pk.value / 1e3
    achieved_tflops = flops_launch / (pair_ms_avg * 1e-3) / 1e12
    traffic = _read_profile_traffic()

    # end to end through the C ABI with host buffers (upload + step + download)
    e2e = run_e2e(sim, w, min(args.steps, 60))
    sim.close()

    if world > 1:
        torch.distributed.barrier()
    if rank != 0:
        return None
    res = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded clusters; no dataset)",
        "config": _config(w, {"parallelism": "replicas" if world > 1 else "single GPU", "mode": "exact"}),
        "impl": "ours",
        "e2e": e2e,
        "gpu_launches": gpu_launches,
        "roofline": {"bound": "fp64", "kernel": "pair_tile_kernel", "achieved": achieved_tflops,
                     "peak": peak_tflops, "unit": "TFLOP/s", "frac": achieved_tflops / peak_tflops,
                     "traffic": traffic,
                     "peak_source": "measured live: FP64 FMA chains (sl_diag_fp64_peak), 2 flops per FMA",
                     "flops_per_launch": flops_launch, "pair_ms_per_launch": pair_ms_avg,
                     "rowsum_ms_per_launch": rowsum_ms / launches,
                     "flop_convention": "add/sub/mul/div/sqrt = 1 flop each (spacelab_gb300/flops.py); "
                                        "div and sqrt cost ~7.5 FMA on this GPU",
                     "contacts": contacts},
        "clocks": clk,
    }
    return res


def _read_profile_traffic():
    """DRAM bytes per pair-kernel launch from the committed ncu summary."""
    p = ROOT / "profiles" / "pair_tile_kernel_n5000.json"
    if p.exists():
        try:
            return json.loads(p.read_text()).get("dram_bytes_per_launch")
        except (OSError, ValueError):
            return None
    return None


def run_e2e(sim, w, steps: int) -> dict:
    """Host-authoritative use of the drop-in: each step uploads the state from
    pinned host buffers, runs sim_one_step on the GPU and downloads it."""
    import ctypes
    import torch
    from spacelab_gb300 import _lib
    lib = _lib.lib()
    n = w.n
    pin = lambda: torch.zeros(3 * n, dtype=torch.float64).pin_memory().numpy()  # noqa: E731
    pos, vel, wv, acc, aacc, prev = (pin() for _ in range(6))
    sim.download()
    pos[:] = sim.group.pos.reshape(-1); vel[:] = sim.group.vel.reshape(-1); wv[:] = sim.group.w.reshape(-1)
    acc[:] = sim.group.acc.reshape(-1); aacc[:] = sim.group.aacc.reshape(-1); prev[:] = pos
    h = sim.handle
    P = _lib.dptr
    e = _lib.Energy()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in range(steps):
        _lib.check(lib.sl_upload_resume(h, P(pos), P(vel), P(wv), P(acc), P(aacc), P(prev)), "sl_upload_resume")
        prev[:] = pos
        _lib.check(lib.sl_step(h, 1, int((k + 1) % w.skip == 0), ctypes.byref(e)), "sl_step")
        _lib.check(lib.sl_download(h, P(pos), P(vel), P(wv), P(acc), P(aacc)), "sl_download")
    el = time.perf_counter() - t0
    return {"value": w.pairs_per_step * steps / el, "unit": UNIT, "h2d_bytes_per_step": 6 * 3 * n * 8,
            "d2h_bytes_per_step": 5 * 3 * n * 8, "steps": steps,
            "api": "sl_upload_resume + sl_step(1) + sl_download per step"}


# ------------------------------------------------------------- reference --
def run_reference(args, rank, world) -> dict | None:
    if rank != 0:
        return None
    from oracle.oracle import ref_available
    w = _workload()
    t0 = time.perf_counter()
    if ref_available():
        # the reference's own sim_one_step (single-threaded by construction)
        r = ref_pin_rate(w, budget_s=30.0)
    else:
        r = cpu_oracle_rate(w, budget_s=30.0, threads=0)
    ms_per_step = w.pairs_per_step / r["value"] * 1e3
    return {"metric": METRIC, "value": r["value"], "unit": UNIT, "n_gpus": 0, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded clusters; no dataset)",
            "config": _config(w, {"parallelism": "host threads"}), "impl": "reference",
            "cpu_baseline": {"value": r["value"], "unit": UNIT, "cores": r["cores"], "kind": r["kind"],
                             "sample": r["sample"]},
            "e2e": {"value": r["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "wall_s": time.perf_counter() - t0}


def main(argv=None) -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--cpu-budget", type=float, default=12.0, help="seconds of CPU oracle timing (rank 0)")
    args = ap.parse_args(argv)
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    rank, world, local_rank = _dist_env()
    if args.impl == "reference":
        res = run_reference(args, rank, world)
        if res is not None:
            print(json.dumps(res), flush=True)
        return 0
    res = run_ours(args, rank, world, local_rank)
    if res is not None:
        sys.path.insert(0, str(ROOT / "tests"))
        res["cpu_baseline"] = cpu_oracle_rate(_workload(), budget_s=args.cpu_budget, threads=0)
        print(json.dumps(res), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
