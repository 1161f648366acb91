"""Multi-process host logic on CPU with the gloo backend (world size 2): bench.py's
max-over-ranks timing and its reference arm, where only rank 0 works and prints; and the
group-sharded SIRT exchange (python/shard.py reduce_df), whose per-group gradients must equal
the single-process ones bit for bit."""
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


def shard_worker(rank, world, port, q):
    """One rank of the group-sharded gradient: the oracle's FP64 gradients of this rank's groups,
    completed by reduce_df over gloo."""
    import numpy as np
    import torch
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    pkg = os.path.join(REPO, "tomographic-image-reconstruction-algorithms_gb300", "python")
    sys.path[:0] = [pkg, os.path.join(REPO, "oracle")]
    import oracle_lib as O
    import shard
    import tomo

    cfg, fo, f = shard_case(tomo)
    meas = O.forward(cfg, fo.astype(np.float64))
    G = O.info(cfg)["n_groups"]
    g0, ng = shard.group_range(G, rank, world)
    corr = torch.full((G, cfg.ny, cfg.nx), float("nan"), dtype=torch.float64)   # other ranks' rows unset
    own, r2 = O.gradient_groups(cfg, f, meas, g0, ng)
    corr[g0:g0 + ng] = torch.from_numpy(own)
    shard.reduce_df(corr)
    r2_all = shard.reduce_resid(r2)
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, corr.numpy().copy(), r2_all))


def shard_case(tomo):
    import numpy as np

    cfg = tomo.cfg_config(nx=48, ny=40, nt=90, n_transducers=20, group_size=4, radius=16.0,
                          cells_per_wavelength=8.0, sponge_width=6)
    y, x = np.mgrid[0:40, 0:48]
    fo = (0.08 * (((x - 22) ** 2 + (y - 19) ** 2) <= 36)).astype(np.float32)
    f = 0.5 * fo.astype(np.float64)
    return cfg, fo, f


def test_group_range_covers_every_group_once():
    sys.path.insert(0, os.path.join(REPO, "tomographic-image-reconstruction-algorithms_gb300", "python"))
    import shard

    for G in (1, 2, 5, 32, 33, 64):
        for world in range(1, min(G, 9) + 1):
            seen = []
            for r in range(world):
                g0, ng = shard.group_range(G, r, world)
                assert ng >= 1
                seen.extend(range(g0, g0 + ng))
            assert seen == list(range(G))
    with pytest.raises(ValueError):
        shard.group_range(3, 0, 4)


@pytest.mark.timeout(300)
def test_gradient_split_over_two_ranks_equals_single_rank():
    """Groups split over two gloo ranks, each rank's per-group gradients from the FP64 oracle,
    completed by reduce_df: every rank holds the single-process per-group gradients bit for bit
    (so any update rule applied to them gives the single-process field), and the summed
    residual matches the single-process one."""
    import numpy as np
    import torch.multiprocessing as mp

    sys.path[:0] = [os.path.join(REPO, "tomographic-image-reconstruction-algorithms_gb300", "python"),
                    os.path.join(REPO, "oracle")]
    import oracle_lib as O
    import tomo

    O.build()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=shard_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted((q.get(timeout=240) for _ in procs), key=lambda t: t[0])
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    cfg, fo, f = shard_case(tomo)
    meas = O.forward(cfg, fo.astype(np.float64))
    want, r2 = O.gradient(cfg, f, meas)
    for rank, corr, r2_all in res:
        assert np.array_equal(corr, want), rank
        assert abs(r2_all - r2) <= 1e-12 * r2
