"""Sharding an ensemble over ranks: LPT bin packing and the result gather.

The multi-process path runs as two `gloo` ranks on the CPU: each rank takes
its LPT share of a drawn ensemble, computes a per-system result on the host
(a checksum of the system's coordinates stands in for its trajectory), and
the gather must return every system exactly once, equal to the serial
computation.  The bench's timing reduction (barrier, max over ranks) runs the
same way.
"""
import os
import socket

import numpy as np
import pytest

from gpucell_gb300.shard import gather_results, lpt_partition, shard_for_rank


def test_lpt_assigns_every_system_once_and_balances():
    rng = np.random.default_rng(0)
    w = np.exp(rng.uniform(np.log(8000), np.log(200000), 64))
    for k in (1, 2, 3, 4, 8):
        parts = lpt_partition(w, k)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(64))
        loads = [w[p].sum() for p in parts]
        lower = max(w.sum() / k, w.max())
        assert max(loads) <= 4.0 / 3.0 * lower + 1e-6
        assert parts == lpt_partition(w, k)           # deterministic
        assert all(p == sorted(p) for p in parts)


def test_lpt_edge_cases():
    assert lpt_partition([], 3) == [[], [], []]
    assert lpt_partition([5.0], 2) == [[0], []]
    assert lpt_partition([1, 1, 1, 1], 2) == [[0, 2], [1, 3]]
    with pytest.raises(ValueError):
        lpt_partition([1.0], 0)
    assert shard_for_rank([3, 2, 1], 0, 1) == [0, 1, 2]
    assert gather_results({1: "a"}, 1) == {1: "a"}


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _checksum(cfg):
    return float(np.float64(cfg.coor).sum()) + cfg.n


def _rank_main(rank, world, port, q):
    import torch.distributed as dist
    from gpucell_gb300 import generator as gen
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    cfgs = gen.ensemble_suite(nsys=6, seed=11, n_range=(2000, 8000), max_cells=2, subdiv=1)
    mine = shard_for_rank([c.n for c in cfgs], rank, world)
    local = {i: _checksum(cfgs[i]) for i in mine}
    merged = gather_results(local, world)
    if rank == 0:
        q.put((sorted(merged.items()), [_checksum(c) for c in cfgs], mine))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_share_an_ensemble():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    merged, serial, mine0 = q.get(timeout=300)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert [k for k, _ in merged] == list(range(6))
    assert [v for _, v in merged] == serial
    assert 0 < len(mine0) < 6


def _rank_times(rank, world, port, q):
    import sys

    import torch
    import torch.distributed as dist
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    if root not in sys.path:
        sys.path.insert(0, root)
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    barrier, max_over_ranks = bench.rank_reducers(world, torch.device("cpu"))
    barrier()
    t = max_over_ranks(10.0 + 5.0 * rank)   # rank 1 is the slower one
    barrier()
    q.put((rank, t))
    dist.destroy_process_group()


def test_bench_times_are_the_max_over_two_gloo_ranks():
    """The bench brackets each timed region with a barrier and reports the
    slowest rank's time, on every rank; one process reduces nothing."""
    import sys

    import torch
    import torch.multiprocessing as mp
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    if root not in sys.path:
        sys.path.insert(0, root)
    import bench
    barrier, max_over_ranks = bench.rank_reducers(1, torch.device("cpu"))
    barrier()
    assert max_over_ranks(3.25) == 3.25
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_times, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=300) for _ in range(2))
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert got == {0: 15.0, 1: 15.0}
