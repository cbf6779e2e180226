"""The N>1 path of bench.py: independent replicas, one per rank, with the
job time taken as the slowest rank's (max over ranks) and the throughput
summed over ranks.  Checked with two gloo ranks on the CPU."""
import os
import socket
import sys
from pathlib import Path

import pytest
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, out):
    sys.path.insert(0, str(ROOT))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms_local = [100.0, 250.0][rank]
    value, ms_max = bench.replica_throughput(1000.0, ms_local, world, device="cpu")
    out.put((rank, value, ms_max))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_replicas_take_the_slowest_rank():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    for rank, value, ms_max in res:
        assert ms_max == 250.0
        assert value == pytest.approx(2 * 1000.0 / 0.25)


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, str(ROOT))
    import bench
    value, ms_max = bench.replica_throughput(500.0, 50.0, 1)
    assert ms_max == 50.0 and value == pytest.approx(10000.0)
