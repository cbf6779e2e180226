"""Benchmark of SpaceLab's step on GB300: pair-interactions/s at N=5000.

Workload: the aggregate collision of a 4000-sphere target and a 1000-sphere
projectile (seeded synthetic clusters; no dataset is involved), FP64, the
reference's write schedule (energy every 100 steps).  One bench step is one
velocity-Verlet step (sim_one_step); a pair interaction is one unordered
pair evaluated per step, N(N-1)/2 per step.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0).  `value` is device-resident throughput (state
in HBM, CUDA events on the library's stream) over steps inside the
collision's impact; `e2e` is the same metric through the C ABI from pinned
host buffers, the state read from them and written back every step
(sl_step_host); `roofline`
reports the pair kernel against the FP64 pipe (exact and mixed) or the FP32
pipe (mixed_df); `cpu_baseline` times the reference's own step (compiled
from its sources, one thread) on a bounded sample on this host.
`--impl reference` times the reference's own step over the same steps.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "pair-interactions/s at N=5000 (FP64 aggregate collision)"
UNIT = "pair-interactions/s"
WORKLOADS = ("aggregate_collision_n5000", "dust_cluster_n1000", "polydisperse_cluster_n20000")


def _dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(
        os.environ.get("LOCAL_RANK", "0"))


def replica_throughput(units_per_rank: float, ms_local: float, world: int, device: str = "cpu") -> tuple[float, float]:
    """Whole-job throughput of `world` independent replicas: every rank did
    `units_per_rank` units in `ms_local` ms; the job takes the slowest rank's
    time.  Returns (units/s over all ranks, max ms).  Uses torch.distributed
    when world > 1 (NCCL on GPUs, gloo on CPU)."""
    ms_max = ms_local
    if world > 1:
        import torch
        import torch.distributed as dist
        t = torch.tensor([ms_local], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms_max = float(t.item())
    return units_per_rank * world / (ms_max * 1e-3), ms_max


def _workload(name: str = "aggregate_collision_n5000"):
    from spacelab_gb300 import configs
    return {"aggregate_collision_n5000": configs.aggregate_collision_5000,
            "dust_cluster_n1000": configs.dust_cluster_1000,
            "polydisperse_cluster_n20000": configs.polydisperse_cluster_20000}[name]()


def _metric(w, mode: str) -> str:
    if w.name == "aggregate_collision_n5000" and mode == "exact":
        return METRIC
    return f"pair-interactions/s at N={w.n} ({'FP64' if mode == 'exact' else 'mixed FP32/FP64'} {w.name})"


L2_BYTES = 129 * 1000 * 1000  # GB300's L2


def working_set_bytes(w, mode: str) -> int:
    """Bytes a step writes and reads back beyond the per-sphere state: the
    exact form's pair-term buffer, or the mixed forms' tile partials and
    contact words per (sphere, partner block)."""
    npad = (w.n + 31) // 32 * 32
    if mode == "exact":
        return 3 * npad * npad * 8
    return (28 if mode == "mixed" else 16) * npad * (npad // 32)


def _config(w, extra=None, mode: str = "exact"):
    ws = working_set_bytes(w, mode) / 1e6
    what = ("the pair-term buffer (3*npad^2 FP64 terms)" if mode == "exact"
            else "tile partials and contact words (no pair-term buffer)")
    if ws * 1e6 > L2_BYTES:
        l2 = (f"per-step working set {ws:.0f} MB of {what}, above the 129 MB L2, written and read every step; "
              f"the timed steps run as one schedule, no flush between them")
    else:
        l2 = (f"per-step working set {ws:.0f} MB of {what}, within the 129 MB L2: each step timed alone, L2 "
              f"flushed between steps by writing a 258 MB buffer outside the timed events")
    cfg = {"workload": w.name, "n_spheres": w.n, "steps_per_write": w.skip,
           "dt_s": w.dt, "kin": w.kin, "kout": w.kout, "seeds": w.info, "l2": l2}
    if w.name == "aggregate_collision_n5000":
        cfg.update({"n_target": 4000, "n_projectile": 1000})
    if extra:
        cfg.update(extra)
    return cfg


# ------------------------------------------------------------------ clocks --
class NvmlClocks:
    """SM clock, maximum SM clock and clock-event (throttle) reasons read
    through NVML (libnvidia-ml, by ctypes) every ~2 ms in a thread, so that
    a timed region of a few tens of milliseconds still gets many samples.
    Read-only: nothing is set."""

    # nvmlClocksEventReason* bits
    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown", 0x40: "hw_thermal_slowdown",
               0x80: "hw_power_brake_slowdown"}

    def __init__(self, device_index: int, pci: tuple[int, int, int] | None = None, period_s: float = 0.002):
        import ctypes
        import threading
        self.ct = ctypes
        self.nvml = ctypes.CDLL("libnvidia-ml.so.1")
        if self.nvml.nvmlInit_v2() != 0:
            raise OSError("nvmlInit failed")
        self.dev = ctypes.c_void_p()
        rc = 1
        if pci is not None:
            bus = f"{pci[0]:08x}:{pci[1]:02x}:{pci[2]:02x}.0".encode()
            rc = self.nvml.nvmlDeviceGetHandleByPciBusId_v2(ctypes.c_char_p(bus), ctypes.byref(self.dev))
        if rc != 0:
            rc = self.nvml.nvmlDeviceGetHandleByIndex_v2(ctypes.c_uint(device_index), ctypes.byref(self.dev))
        if rc != 0:
            raise OSError("no NVML handle for the device")
        self.reason_fn = getattr(self.nvml, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            self.nvml.nvmlDeviceGetCurrentClocksThrottleReasons
        self.period = period_s
        self.samples: list[tuple[int, int, int]] = []
        self._stop = threading.Event()
        self._thread = threading.Thread(target=self._loop, daemon=True)

    def _read(self):
        ct = self.ct
        sm, smax, reasons = ct.c_uint(), ct.c_uint(), ct.c_ulonglong()
        if self.nvml.nvmlDeviceGetClockInfo(self.dev, 1, ct.byref(sm)) != 0:  # NVML_CLOCK_SM
            return None
        self.nvml.nvmlDeviceGetMaxClockInfo(self.dev, 1, ct.byref(smax))
        self.reason_fn(self.dev, ct.byref(reasons))
        return sm.value, smax.value, reasons.value

    def _loop(self):
        while not self._stop.is_set():
            r = self._read()
            if r is not None:
                self.samples.append(r)
            time.sleep(self.period)

    def start(self):
        r = self._read()
        if r is not None:
            self.samples.append(r)
        self._thread.start()

    def stop(self) -> dict:
        self._stop.set()
        self._thread.join(timeout=2)
        r = self._read()
        if r is not None:
            self.samples.append(r)
        self.nvml.nvmlShutdown()
        return self.summarize(self.samples)

    @classmethod
    def summarize(cls, samples) -> dict:
        if not samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"], "source": "nvml"}
        sm = [a for a, _, _ in samples]
        reasons = sorted({name for _, _, bits in samples for bit, name in cls.REASONS.items() if bits & bit})
        return {"sm_mhz": float(np.median(sm)), "sm_min_mhz": float(min(sm)),
                "sm_max_mhz": float(max(b for _, b, _ in samples)), "reasons": reasons, "samples": len(samples),
                "source": "nvml, every ~2 ms over the timed region"}


def clock_sampler(local_rank: int):
    """NVML sampler for the current CUDA device, else nvidia-smi."""
    try:
        import torch
        p = torch.cuda.get_device_properties(local_rank)
        pci = (int(p.pci_domain_id), int(p.pci_bus_id), int(p.pci_device_id))
    except Exception:
        pci = None
    try:
        return NvmlClocks(local_rank, pci)
    except (OSError, AttributeError):
        return ClockSampler(local_rank)


class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    # SL_CLOCKS_DIR: where the raw nvidia-smi samples are kept (default: a
    # temporary file, removed after it is summarised).
    def __init__(self, gpu_index: int):
        self.proc = None
        self.gpu = gpu_index
        keep = os.environ.get("SL_CLOCKS_DIR")
        if keep:
            self.path = Path(keep) / f"clocks_rank{gpu_index}.csv"
            self.keep = True
        else:
            fd, name = tempfile.mkstemp(prefix=f"sl_clocks{gpu_index}_", suffix=".csv")
            os.close(fd)
            self.path = Path(name)
            self.keep = False

    def start(self):
        try:
            self.path.parent.mkdir(parents=True, exist_ok=True)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.fh,
                                         stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            if not self.keep:
                self.path.unlink(missing_ok=True)
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.fh.close()
        text = self.path.read_text()
        if not self.keep:
            self.path.unlink(missing_ok=True)
        return self.summarize(text)

    @staticmethod
    def summarize(text: str) -> dict:
        """Median and maximum SM clock and the throttle reasons seen in
        nvidia-smi CSV samples of FIELDS (no header, no units)."""
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in text.splitlines():
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
def port_state_at(w, step: int, threads: int = 0):
    """The workload's state after `step` steps of its schedule (write steps
    every w.skip), computed by the row-parallel CPU oracle -- bit-identical
    to the reference's own step.  Returns the oracle object (its state is
    the end of that step)."""
    from oracle.oracle import CpuOracle
    g = w.group
    o = CpuOracle(g.pos, g.vel, g.w, g.R, g.m, g.moi, w.material, w.dt, w.kin, w.kout)
    o.init()
    for s in range(1, step + 1):
        o.step(s % w.skip == 0, threads=threads)
    return o


def _timed_steps(step_fn, first: int, skip: int, steps: int | None, budget_s: float | None) -> tuple[int, float]:
    """Run step_fn(write) for the schedule's steps first, first+1, ...:
    exactly `steps` of them, or (steps None) until budget_s has passed and
    at least 2 ran.  Returns (steps run, seconds)."""
    t0 = time.perf_counter()
    k = 0
    while True:
        step_fn((first + k) % skip == 0)
        k += 1
        el = time.perf_counter() - t0
        if (steps is not None and k >= steps) or (steps is None and k >= 2 and el >= budget_s):
            return k, el


def cpu_oracle_rate(w, budget_s: float | None, threads: int = 0, start=None, first: int = 1,
                    steps: int | None = None, warmup: int = 1) -> dict:
    """Row-parallel CPU oracle (the C restatement) on `threads` host threads
    (0 = all): `warmup` untimed steps, then `steps` timed steps or, with
    steps None, steps until budget_s has passed.  start: an oracle whose
    state to continue from (else the workload's initial state)."""
    from oracle.oracle import CpuOracle
    g = w.group
    o = start
    if o is None:
        o = CpuOracle(g.pos, g.vel, g.w, g.R, g.m, g.moi, w.material, w.dt, w.kin, w.kout)
        o.init()
    for k in range(warmup):
        o.step((first + k) % w.skip == 0, threads=threads)
    n, el = _timed_steps(lambda wr: o.step(wr, threads=threads), first + warmup, w.skip, steps, budget_s)
    cores = CpuOracle.max_threads() if threads == 0 else threads
    return {"value": w.pairs_per_step * n / el, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"{n} steps from step {first + warmup} of the N={w.n} workload ({el:.2f} s), row-parallel C "
                      f"restatement of sim_one_step (bit-identical to the reference build; restatement, not "
                      f"reference), {cores} threads, {os.uname().machine} host"}


def ref_pin_rate(w, budget_s: float | None, native: bool = False, start_state=None, first: int = 1,
                 steps: int | None = None, warmup: int = 1) -> dict:
    """The reference's own sim_one_step (oracle/_ref, compiled from the
    reference's sources), one thread -- the reference's step is
    single-threaded: `warmup` untimed steps, then `steps` timed steps or,
    with steps None, steps until budget_s has passed.  start_state:
    (pos, vel, w, acc, aacc) at the end of step first-1 (else the
    workload's initial state)."""
    from oracle.oracle import RefPin
    g = w.group
    ref = RefPin(g.pos, g.vel, g.w, g.R, g.m, g.moi, w.dt, w.kin, w.kout, native=native)
    if start_state is not None:
        ref.resume(*start_state)
    for k in range(warmup):
        ref.step((first + k) % w.skip == 0)
    n, el = _timed_steps(ref.step, first + warmup, w.skip, steps, budget_s)
    flags = "-O3 -march=native, contraction allowed" if native else "-O2 -ffp-contract=off"
    return {"value": w.pairs_per_step * n / el, "unit": UNIT, "cores": 1, "kind": "reference",
            "sample": f"{n} steps from step {first + warmup} of the N={w.n} workload ({el:.2f} s), the "
                      f"reference's sim_one_step compiled from its sources ({flags}), 1 thread, "
                      f"{os.uname().machine} host"}


def cpu_baselines(w, budget_s: float) -> tuple[dict, list[dict]]:
    """Rank 0's cpu_baseline (the reference's own step on 1 thread where it
    was built, else the port on all cores) and the secondary lines, each on
    a bounded sample from the workload's initial state (the CPU's cost per
    step does not depend on how many pairs touch: contacts are O(N) of the
    N(N-1)/2 pairs)."""
    from oracle.oracle import ref_available
    lines = []
    if ref_available():
        primary = ref_pin_rate(w, budget_s)
        if ref_available(native=True):
            lines.append(ref_pin_rate(w, budget_s / 2, native=True))
        lines.append(cpu_oracle_rate(w, budget_s / 2, threads=0))
    else:
        primary = cpu_oracle_rate(w, budget_s, threads=0)
    return primary, lines


# ------------------------------------------------------------------ ours --
def default_start_step(w) -> int:
    """First step of the measured window minus one.  The aggregate collision
    is measured after its clusters have met (they touch after ~1500 of its
    5000 steps), so that contact pairs, the spring switch and friction are
    in the timed steps; the other workloads from their start."""
    return 2500 if w.name == "aggregate_collision_n5000" else 0



def run_ours(args, rank, world, local_rank) -> dict | None:
    import torch
    torch.cuda.set_device(local_rank)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from spacelab_gb300 import GpuStep, _lib
    from spacelab_gb300 import flops as F

    w = _workload(args.workload)
    g = w.group
    sim = GpuStep(g.copy(), w.material, args.mode)
    if args.overlap:
        sim.set_overlap(True)
    if args.mode == "exact":
        sim.set_rowsum(args.rowsum)
    sim.set_scalars(w.dt, w.kin, w.kout)
    sim.init_conditions()
    stream = torch.cuda.ExternalStream(sim.stream_ptr())

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
            torch.cuda.synchronize()

    # advance to the start of the measured window on the GPU (untimed; the
    # schedule's write steps included), then warm up (the kernels of both
    # step kinds are loaded by the write steps of the advance or by the
    # first sl_run)
    start = default_start_step(w) if args.start_step is None else args.start_step
    if start > 0:
        sim.sim_looper(steps=start + 1, skip=w.skip)
    contacts_start = int(len(sim.contacts()))
    sim.sim_looper(steps=start + 1 + args.warmup, skip=w.skip, first_step=start + 1)
    first = start + 1 + args.warmup
    nwrites = sum(1 for s in range(first, first + args.steps) if s % w.skip == 0)

    # Inputs larger than L2 (the exact form's pair-term buffer) are timed as
    # one run of the schedule.  Where the per-step working set fits in L2
    # (the mixed forms at small N), each step is timed alone and L2 is
    # flushed between steps by writing a buffer larger than it, outside the
    # timed events.
    flush = None if working_set_bytes(w, args.mode) > L2_BYTES else \
        torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device="cuda")
    clocks = clock_sampler(local_rank)
    barrier()
    clocks.start()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    if flush is None:
        ev0.record(stream)
        sim.sim_looper(steps=first + args.steps, skip=w.skip, first_step=first)
        ev1.record(stream)
        barrier()
        ms = ev0.elapsed_time(ev1)
    else:
        ms = 0.0
        with torch.cuda.stream(stream):
            for k in range(args.steps):
                flush.fill_(float(k))
                ev0.record(stream)
                sim.step(1, write_last=(first + k) % w.skip == 0)
                ev1.record(stream)
                ev1.synchronize()
                ms += ev0.elapsed_time(ev1)
        barrier()
    clk = clocks.stop()
    contacts_end = int(len(sim.contacts()))
    value, ms_max = replica_throughput(w.pairs_per_step * args.steps, ms, world, device="cuda")
    gpu_launches = sim.step_launches(False) * (args.steps - nwrites) + sim.step_launches(True) * nwrites
    pair_launches = (sim.step_launches(False) - 1) // 2
    next_step = first + args.steps

    # per-step timing of the pair pass (non-write steps), same stream: with
    # the pipelined exact step the pair span holds all pair phases and the
    # row sums that run beside them; "rowsum" is the exposed remainder
    sim.kernel_timing(True)
    nk = max(10, min(50, args.steps))
    sim.step(nk, write_last=False)
    next_step += nk
    pair_ms, rowsum_ms, launches = sim.kernel_times(reset=True)
    sim.kernel_timing(False)
    contacts = int(len(sim.contacts()))
    pair_ms_avg = pair_ms / launches  # one record per step
    flops_launch = F.pair_flops(w.pairs_per_step, contacts, write=False)
    import ctypes
    lib = _lib.lib()
    nsm = torch.cuda.get_device_properties(local_rank).multi_processor_count
    sm_max = (clk.get("sm_max_mhz") or 2070.0) * 1e6
    pk = ctypes.c_double()
    if args.mode in ("exact", "mixed"):
        # both run on the FP64 pipe: the exact form's pair arithmetic, and
        # the mixed form's 9 FP64 adds per pair (r, and the two spheres'
        # FP64 sums), one FP64 lane-op each
        peak_fn = "sl_diag_fp64_peak"
        _lib.check(lib.sl_diag_fp64_peak(ctypes.byref(pk)), peak_fn)
        if args.mode == "exact":
            work, unit = flops_launch, "TFLOP/s"
            peak = pk.value / 1e3
            peak_source = "measured live: FP64 FMA chains (sl_diag_fp64_peak), 2 flops per FMA"
            nominal = nsm * 2 * 2 * sm_max / 1e12
            nominal_source = f"{nsm} SMs x 2 FP64 FMA/clock x 2 flops x {sm_max / 1e6:.0f} MHz"
            bound = "fp64"
        else:
            work, unit = F.MIXED64_FP64_OPS_PER_PAIR * w.pairs_per_step, "T FP64 lane-ops/s"
            peak = pk.value / 2 / 1e3
            peak_source = "measured live: FP64 FMA chains (sl_diag_fp64_peak), one lane-op per FMA"
            nominal = nsm * 2 * sm_max / 1e12
            nominal_source = f"{nsm} SMs x 2 FP64 lane-ops/clock x {sm_max / 1e6:.0f} MHz"
            bound = "fp64 (adds)"
    else:
        peak_fn = "sl_diag_fp32_peak"
        _lib.check(lib.sl_diag_fp32_peak(ctypes.byref(pk)), peak_fn)
        work, unit = flops_launch, "TFLOP/s"
        peak = pk.value / 1e3
        peak_source = "measured live: FP32 FMA chains (sl_diag_fp32_peak), 2 flops per FMA"
        nominal = nsm * 128 * 2 * sm_max / 1e12
        nominal_source = f"{nsm} SMs x 128 FP32 FMA/clock x 2 flops x {sm_max / 1e6:.0f} MHz"
        bound = "fp32"
    # latency of a dependent FP64 add chain (bounds the row sums)
    chain = {}
    for wps in (1, 4):
        cy = ctypes.c_double()
        _lib.check(lib.sl_diag_fp64_add_latency(wps, 32, ctypes.byref(cy)), "sl_diag_fp64_add_latency")
        chain[f"{wps}_warps_per_sm"] = cy.value
    achieved = work / (pair_ms_avg * 1e-3) / 1e12
    traffic = _read_profile_traffic() if (args.mode == "exact" and w.name == "aggregate_collision_n5000") else None

    # the schedule's write steps (every w.skip steps; none may fall in a short
    # timed window): one write step timed alone, on the library's stream, and
    # the per-step average of the schedule (skip - 1 plain steps, one write)
    wev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    write_ms = []
    for _ in range(3):
        wev[0].record(stream)
        sim.step(1, write_last=True)
        wev[1].record(stream)
        torch.cuda.synchronize()
        write_ms.append(wev[0].elapsed_time(wev[1]))
    next_step += 3
    write_step_ms = float(np.median(write_ms))
    plain_ms = ms_max / args.steps if nwrites == 0 else None
    schedule = None
    if plain_ms is not None:
        sched_ms = ((w.skip - 1) * plain_ms + write_step_ms) / w.skip
        schedule = {"write_step_ms": write_step_ms, "plain_step_ms": plain_ms, "ms_per_step": sched_ms,
                    "value": w.pairs_per_step * world / (sched_ms * 1e-3),
                    "how": f"one write step every {w.skip} steps: ({w.skip - 1} x plain + 1 x write) / {w.skip}"}

    # end to end through the C ABI with host buffers (upload + step + download)
    e2e = run_e2e(sim, w, min(args.steps, 60), first_step=next_step)
    pair_kernel = sim.pair_kernel()
    sim.close()

    if world > 1:
        torch.distributed.barrier()
    if rank != 0:
        return None
    res = {
        "metric": _metric(w, args.mode), "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64" if args.mode == "exact" else "f32+f64",
        "data": "synthetic (seeded clusters; no dataset)",
        "config": _config(w, {"parallelism": "replicas" if world > 1 else "single GPU", "mode": args.mode,
                               "overlap": bool(args.overlap), "start_step": start,
                               **({"rowsum": args.rowsum} if args.mode == "exact" else {}),
                               "timed_steps": [first, first + args.steps - 1], "write_steps_timed": nwrites,
                               "contacts_at_start_step": contacts_start,
                               "contacts_after_timed_steps": contacts_end}, mode=args.mode),
        "impl": "ours",
        "e2e": e2e,
        "schedule_average": schedule,
        "gpu_launches": gpu_launches,
        "roofline": {"bound": bound,
                     "kernel": pair_kernel,
                     "achieved": achieved,
                     "peak": peak, "unit": unit, "frac": achieved / peak,
                     "traffic": traffic,
                     "peak_source": peak_source,
                     "peak_nominal": nominal, "frac_of_nominal": achieved / nominal,
                     "peak_nominal_source": nominal_source,
                     "flops_per_step": flops_launch, "pair_ms_per_step": pair_ms_avg,
                     "rowsum_exposed_ms_per_step": rowsum_ms / launches,
                     "fp64_add_chain_cycles": chain,
                     "pair_launches_per_step": pair_launches,
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


def run_e2e(sim, w, steps: int, first_step: int = 1) -> dict:
    """Host-authoritative use of the drop-in: every step reads the state from
    pinned host buffers, runs sim_one_step on the GPU and writes the new state
    back into them (sl_step_host: the exchange and the step in one call, one
    wait for the GPU)."""
    import ctypes
    import torch
    from spacelab_gb300 import _lib
    lib = _lib.lib()
    n = w.n
    pin = lambda: torch.zeros(3 * n, dtype=torch.float64).pin_memory().numpy()  # noqa: E731
    pos, vel, wv, acc, aacc = (pin() for _ in range(5))
    sim.download()
    pos[:] = sim.group.pos.reshape(-1); vel[:] = sim.group.vel.reshape(-1); wv[:] = sim.group.w.reshape(-1)
    acc[:] = sim.group.acc.reshape(-1); aacc[:] = sim.group.aacc.reshape(-1)
    h = sim.handle
    # the host buffers stay put: their pointers are formed once, as a C
    # caller would hold them.  The state is the end of a step, so the
    # previous-step positions that choose kin/kout are the current ones, as
    # the reference's `distances` hold the pair distances of the current
    # positions between steps.
    P = _lib.dptr
    pp, pv, pw, pa, paa = P(pos), P(vel), P(wv), P(acc), P(aacc)
    e = _lib.Energy()
    pe = ctypes.byref(e)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in range(steps):
        _lib.check(lib.sl_step_host(h, pp, pv, pw, pa, paa, int((first_step + k) % w.skip == 0), pe),
                   "sl_step_host")
    el = time.perf_counter() - t0
    return {"value": w.pairs_per_step * steps / el, "unit": UNIT, "h2d_bytes_per_step": 5 * 3 * n * 8,
            "d2h_bytes_per_step": 5 * 3 * n * 8, "steps": steps, "first_step": first_step,
            "api": "sl_step_host per step: reads pos, vel, w, acc, aacc from pinned host arrays, steps, writes them back"}


# ------------------------------------------------ FP64 add-chain latency --
def run_fp64_latency_table() -> dict:
    """Cycles per dependent FP64 add (sl_diag_fp64_add_latency) for 1-8
    warps per SM and 8-32 active lanes per warp: what bounds the exact row
    sums' chains."""
    import ctypes
    import torch
    from spacelab_gb300 import _lib
    torch.cuda.init()
    lib = _lib.lib()
    c = ctypes.c_double()
    rows = []
    for warps in (1, 2, 3, 4, 5, 6, 8):
        for lanes in (8, 16, 24, 32):
            _lib.check(lib.sl_diag_fp64_add_latency(warps, lanes, ctypes.byref(c)), "sl_diag_fp64_add_latency")
            rows.append({"warps_per_sm": warps, "active_lanes": lanes, "cycles_per_add": round(c.value, 1),
                         "lane_adds_per_clock_per_sm": round(warps * lanes / c.value, 3)})
    return {"metric": "FP64 dependent-add latency", "unit": "cycles per add at the rated SM clock", "table": rows,
            "gpu": torch.cuda.get_device_name(0)}


# --------------------------------------------------- mixed vs FP64 report --
def run_drift(args) -> dict:
    """Both mixed-precision forms against the FP64 form on the same seed:
    energy drift |E(t) - E(0)| / |E(0)| of each run, each mixed run's
    energy difference from the FP64 run at every write step, the final
    position and velocity error, and every run's throughput (wall clock of
    the whole schedule, write steps and host syncs included)."""
    import torch
    from spacelab_gb300 import GpuStep
    w = _workload(args.workload)
    out = {"metric": f"mixed vs FP64 on {w.name}", "workload": w.name, "n_spheres": w.n, "steps": args.drift_steps,
           "steps_per_write": w.skip}
    runs = {}
    for mode in ("exact", "mixed", "mixed_df"):
        sim = GpuStep(w.group.copy(), w.material, mode)
        sim.set_scalars(w.dt, w.kin, w.kout)
        e0 = sim.init_conditions()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        rows = sim.sim_looper(steps=args.drift_steps + 1, skip=w.skip)
        el = time.perf_counter() - t0
        g = sim.download()
        runs[mode] = {"E0": e0.PE + e0.KE, "E": np.array([r.E for r in rows]), "pos": g.pos.copy(),
                      "vel": g.vel.copy(), "pairs_per_s": w.pairs_per_step * args.drift_steps / el,
                      "kernel": sim.pair_kernel()}
        sim.close()
    ex = runs["exact"]
    E0 = abs(ex["E0"])
    out["energy_drift_fp64"] = float(np.abs(ex["E"] - ex["E0"]).max() / E0)
    out["pairs_per_s_fp64"] = ex["pairs_per_s"]
    for mode in ("mixed", "mixed_df"):
        mx = runs[mode]
        out[mode] = {
            "pair_kernel": mx["kernel"],
            "energy_drift": float(np.abs(mx["E"] - mx["E0"]).max() / E0),
            "energy_minus_fp64": float(np.abs(mx["E"] - ex["E"]).max() / E0),
            "pos_err_rel_to_size": float(np.abs(mx["pos"] - ex["pos"]).max() / np.abs(ex["pos"]).max()),
            "pos_err_rel_to_radius": float(np.abs(mx["pos"] - ex["pos"]).max() / float(w.group.R.max())),
            "vel_err_rel_to_max": float(np.abs(mx["vel"] - ex["vel"]).max() / np.abs(ex["vel"]).max()),
            "pairs_per_s": mx["pairs_per_s"],
            "speedup_over_fp64": mx["pairs_per_s"] / ex["pairs_per_s"],
        }
    out["mixed_df_over_mixed"] = runs["mixed_df"]["pairs_per_s"] / runs["mixed"]["pairs_per_s"]
    return out


# ------------------------------------------------------ batched collisions --
def run_batched(args) -> dict:
    """Collisions/s of the batched solver (one persistent launch over the
    whole sweep, autotuned shape) next to the same kind of collisions run
    one at a time through the single-system step: a size-stratified sample
    of --baseline-instances collisions (evenly spaced quantiles of the
    sphere count), scaled to the whole sweep."""
    import torch
    from spacelab_gb300 import batch as B
    torch.cuda.init()
    t0 = time.perf_counter()
    cols = B.sample_collisions(args.batched, seed=3, nt_range=(args.nt_min, args.nt_max))
    build_s = time.perf_counter() - t0
    steps = args.batch_steps
    run = B.BatchRun(cols, args.mode, steps=steps, skip=100)
    tuned = run.autotune(sample_steps=8)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ev0.record()
    wall = run.run(1, steps, do_init=True)
    ev1.record()
    torch.cuda.synchronize()
    bad = int(run.status().sum())
    touched = B.made_contact(run.energy())
    counts = np.array([c.n for c in cols])
    pair_evals = float((counts.astype(np.float64) * (counts - 1) / 2).sum()) * steps
    idx = B.stratified_indices(cols, args.baseline_instances)
    sample = [cols[i] for i in idx]
    k = len(sample)
    base_s, _ = B.run_per_instance(sample, steps, 100, args.mode)
    base_rate = k / base_s
    step_s = B.run_per_instance_steps(sample, steps, 100, args.mode)
    step_rate = k / step_s
    rate = len(cols) / wall
    how = (f"{k} collisions at evenly spaced quantiles of the sphere count ({int(counts[idx].min())}-"
           f"{int(counts[idx].max())} spheres, {int(touched[idx].sum())} of them made contact), one after another")
    return {"metric": f"batched collisions/s ({len(cols)} collisions, {steps} steps each, {args.mode})",
            "value": rate, "unit": "collisions/s", "higher_is_better": True, "impl": "ours",
            "collisions": len(cols), "steps_per_collision": steps, "spheres_total": int(counts.sum()),
            "spheres_per_collision": [int(counts.min()), int(counts.max())],
            "collisions_with_contact": int(touched.sum()),
            "contact_criterion": "E = PE + KE fell by more than 1e-3 of the initial KE (dissipation needs contact)",
            "wall_s": wall, "pair_interactions_per_s": pair_evals / wall, "nonfinite_instances": bad,
            "autotune": tuned,
            "per_instance_baseline": {"collisions": k, "seconds": base_s, "collisions_per_s": base_rate,
                                      "how": how + ", sl_run per instance (graph per write interval)"},
            "per_step_launch_baseline": {"collisions": k, "seconds": step_s, "collisions_per_s": step_rate,
                                         "how": how + ", sl_step(1) per step (the sim_one_step drop-in)"},
            "speedup_over_per_instance": rate / base_rate, "speedup_over_per_step_launches": rate / step_rate,
            "build_s": build_s, "k_speed_div": 50.0,
            "dtype": "f64" if args.mode == "exact" else "f32+f64",
            "data": "synthetic (seeded collision sweep; no dataset)"}


# -------------------------------------------------------- surrogate study --
def run_surrogate_study(args) -> dict:
    """Train the 5-member BF16 MLP ensemble on collisions of the batched
    solver's sweep, choose the screening threshold on held-out validation
    collisions for a stated error target, screen a parameter sweep, re-run
    uncertain points plus a random audit with the simulator, and account
    the cost."""
    import torch
    from spacelab_gb300 import batch as B
    from spacelab_gb300 import surrogate as S
    from spacelab_gb300 import sweep as W
    torch.cuda.init()
    steps = args.study_steps
    t0 = time.perf_counter()
    data = B.sample_collisions(args.train_collisions, seed=21, nt_range=W.NT_RANGE, clearance=W.CLEARANCE,
                               k_speed_div=W.K_SPEED_DIV)
    build_s = time.perf_counter() - t0
    y, sim_info = W.simulate(data, steps, mode="mixed_df")
    x = W.features(data)
    perm = np.random.default_rng(24).permutation(len(data))
    nval = max(1, len(data) // 10)
    val, trn = perm[:nval], perm[nval:]
    ens = S.Ensemble(8, 4, members=5, seed=3)
    fit = ens.fit(x[trn], y[trn], epochs=args.epochs, batch=256, lr=1e-3)
    targets = sorted({0.15, 0.175, 0.2, 0.25, 0.3, args.error_target})
    curve = {str(t): W.pick_threshold(ens, x[val], y[val], t) for t in targets}
    chosen = curve[str(args.error_target)]
    points = W.sample_params(args.sweep_points, seed=22)
    res = W.screen_sweep(ens, points, steps, threshold=chosen["threshold"], audit=args.audit, seed=23,
                         sim_mode="mixed_df", fp64_check=args.fp64_check)
    # the method without the network: predict the training mean everywhere
    mean_pred = (np.abs(y[trn].mean(0) - y[val]).mean(0) / ens.ys).tolist()
    return {"metric": "surrogate-screened sweep cost ratio (simulating every point / screened)",
            "value": res["cost_ratio"], "unit": "x", "higher_is_better": True,
            "outcome_error": f"mean absolute error of accepted validation points <= {args.error_target} x each "
                             f"outcome's spread",
            "train_collisions": len(trn), "validation_collisions": len(val), "steps_per_collision": steps,
            "train_sim_s": sim_info["seconds"], "train_sim_pairs_per_s": sim_info["pair_evals"] / sim_info["seconds"],
            "train_nonfinite": sim_info["nonfinite"], "build_s": build_s,
            "fit_s": fit["seconds"], "final_loss": fit["final_loss"], "outcomes": list(S.OUTCOMES),
            "outcome_spread": ens.ys.tolist(),
            "threshold_by_validation": curve, "chosen": chosen,
            "validation_mae_std_units_without_network": mean_pred,
            "screen": res,
            "recipe": {"nt_range": list(W.NT_RANGE), "clearance": "centres 1.1 (Rt+Rp) apart",
                       "k_speed_div": W.K_SPEED_DIV, "simulator": "batched solver, mixed_df"},
            "data": "synthetic (seeded collision sweep; no dataset)"}


# ------------------------------------------------------------- reference --
def run_reference(args, rank, world) -> dict | None:
    """The reference arm: the reference's own sim_one_step (oracle/_ref,
    compiled from its sources; single-threaded, as the reference is) over
    the same steps of the same workload as the GPU arm -- W warm-up steps,
    then exactly K timed steps from the same start step.  The state at the
    start step is made by the row-parallel oracle (bit-identical to the
    reference's step), untimed.  Secondary lines: the reference at -O3
    -march=native, and the oracle restatement on all host cores."""
    if rank != 0:
        return None
    from oracle.oracle import ref_available
    w = _workload(args.workload)
    t0 = time.perf_counter()
    start = default_start_step(w) if args.start_step is None else args.start_step
    o = port_state_at(w, start) if start > 0 else None
    state = None
    if o is not None:
        st = o.state()
        state = tuple(st[k] for k in ("pos", "vel", "w", "acc", "aacc"))
    timing = dict(first=start + 1, steps=args.steps, warmup=args.warmup)
    secondary = []
    if ref_available():
        r = ref_pin_rate(w, None, start_state=state, **timing)
        if ref_available(native=True):
            secondary.append(ref_pin_rate(w, None, native=True, start_state=state, **timing))
        secondary.append(cpu_oracle_rate(w, None, threads=0, start=o, **timing))
    else:
        r = cpu_oracle_rate(w, None, threads=0, start=o, **timing)
    ms_per_step = w.pairs_per_step / r["value"] * 1e3
    first = start + 1 + args.warmup
    cfg = _config(w, {"parallelism": "host threads", "start_step": start,
                      "timed_steps": [first, first + args.steps - 1],
                      "write_steps_timed": sum(1 for s in range(first, first + args.steps) if s % w.skip == 0)})
    return {"metric": METRIC, "value": r["value"], "unit": UNIT, "n_gpus": 0, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded clusters; no dataset)",
            "config": cfg, "impl": "reference",
            "cpu_baseline": {"value": r["value"], "unit": UNIT, "cores": r["cores"], "kind": r["kind"],
                             "sample": r["sample"]},
            "cpu_baselines_secondary": secondary,
            "e2e": {"value": r["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "wall_s": time.perf_counter() - t0}


def main(argv=None) -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--cpu-budget", type=float, default=12.0, help="seconds of CPU baseline timing (rank 0)")
    ap.add_argument("--start-step", type=int, default=None,
                    help="steps of the schedule run before warm-up and the timed steps (default: 2500 for the "
                         "aggregate collision, after its clusters have met; 0 otherwise)")
    ap.add_argument("--mode", choices=["exact", "mixed", "mixed_df"], default="exact",
                    help="exact: FP64, bit-identical to the reference; mixed: FP32 force arithmetic with FP64 "
                         "displacements, overlaps and accumulation; mixed_df: the double-float variant "
                         "(--batched runs exact or mixed_df)")
    ap.add_argument("--overlap", action="store_true",
                    help="exact mode: run the row sums beside the pair phases (sl_set_overlap)")
    ap.add_argument("--rowsum", choices=["int", "fp64"], default="fp64",
                    help="exact mode: the row sums' FP64 additions on the FP64 unit (default) or the integer pipe "
                         "(sl_set_rowsum); identical results")
    ap.add_argument("--workload", choices=WORKLOADS, default="aggregate_collision_n5000")
    ap.add_argument("--fp64-latency-table", action="store_true",
                    help="print the dependent FP64 add latency for 1-8 warps per SM and 8-32 active lanes")
    ap.add_argument("--drift-steps", type=int, default=0,
                    help="instead of the benchmark: run the mixed and the FP64 form side by side for this many "
                         "steps and report energy drift and trajectory error")
    ap.add_argument("--batched", type=int, default=0,
                    help="instead of the benchmark: this many sampled collisions through the batched solver")
    ap.add_argument("--batch-steps", type=int, default=300)
    ap.add_argument("--baseline-instances", type=int, default=64)
    ap.add_argument("--surrogate-study", action="store_true",
                    help="instead of the benchmark: train the surrogate ensemble and screen a sweep")
    ap.add_argument("--train-collisions", type=int, default=50000)
    ap.add_argument("--sweep-points", type=int, default=1000000)
    ap.add_argument("--study-steps", type=int, default=3000)
    ap.add_argument("--epochs", type=int, default=150)
    ap.add_argument("--error-target", type=float, default=0.2,
                    help="surrogate study: mean absolute error of the accepted validation points, in units of "
                         "each outcome's spread, that sets the screening threshold")
    ap.add_argument("--audit", type=float, default=0.01)
    ap.add_argument("--fp64-check", type=int, default=64,
                    help="surrogate study: audit points also re-run with the FP64 exact method")
    ap.add_argument("--nt-min", type=int, default=64)
    ap.add_argument("--nt-max", type=int, default=1600)
    args = ap.parse_args(argv)
    # at least 3 untimed warm-up steps: a smaller request is raised, and the
    # line's "warmup" reports the steps actually run
    warmup_requested = args.warmup
    args.warmup = max(args.warmup, 3)
    rank, world, local_rank = _dist_env()

    def emit(res):
        if warmup_requested != args.warmup:
            res["warmup_requested"] = warmup_requested
        print(json.dumps(res), flush=True)

    if args.impl == "reference":
        res = run_reference(args, rank, world)
        if res is not None:
            emit(res)
        return 0
    if args.fp64_latency_table:
        emit(run_fp64_latency_table())
        return 0
    if args.drift_steps:
        emit(run_drift(args))
        return 0
    if args.batched:
        emit(run_batched(args))
        return 0
    if args.surrogate_study:
        emit(run_surrogate_study(args))
        return 0
    res = run_ours(args, rank, world, local_rank)
    if res is not None:
        res["cpu_baseline"], res["cpu_baselines_secondary"] = cpu_baselines(_workload(args.workload),
                                                                           budget_s=args.cpu_budget)
        emit(res)
    return 0


if __name__ == "__main__":
    sys.exit(main())
