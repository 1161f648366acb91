"""The multi-process host logic of bench.py on CPU with the gloo backend (world size 2):
max-over-ranks timing and the reference arm, where only rank 0 works and prints."""
import io
import os
import socket
import sys
from contextlib import redirect_stdout

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def worker(rank, world, port, q):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sys.path.insert(0, REPO)
    import bench

    m = bench.max_over_ranks(1.0 + rank, dist)
    args = type("A", (), {"steps": 1, "warmup": 1, "workload": "c1"})()
    out = io.StringIO()
    if rank != 0:
        with redirect_stdout(out):
            bench.reference_arm(args, bench.WORKLOADS["c1"], rank, world)
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, m, out.getvalue()))


@pytest.mark.timeout(300)
def test_max_over_ranks_and_reference_arm_rank_gating():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=240) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [m for _, m, _ in res] == [2.0, 2.0]
    assert res[1][2] == ""          # rank 1 of the reference arm does no work and prints nothing
