"""World-size-2 gloo tests of the multi-GPU host logic on CPU: network sharding covers
every network exactly once with balanced work, max/sum over ranks, and the gather of
per-network log-norms (the only cross-rank exchange of the batched workload)."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, sizes, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import sys
        sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                                        "itensornetworksnext.jl_gb300"))
        from itn_gb300 import distributed as D
        lo, hi = D.shard_networks(sizes, rank, world)
        local = {k: float(k) * 0.5 - 3.0 for k in range(lo, hi)}  # stand-in log-norms
        logz = D.gather_logz(local, len(sizes))
        t = D.max_over_ranks(1.0 + rank)
        work = D.sum_over_ranks(float(sum(sizes[lo:hi])))
        out[rank] = (lo, hi, logz.tolist(), t, work)
    finally:
        dist.destroy_process_group()


def test_shard_and_reduce_world2():
    rng = np.random.default_rng(0)
    sizes = rng.integers(16, 257, size=37).tolist()
    world = 2
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    port = _free_port()
    mp.start_processes(_worker, args=(world, port, sizes, out), nprocs=world, join=True,
                       start_method="spawn")
    res = [out[r] for r in range(world)]
    ranges = [(lo, hi) for lo, hi, *_ in res]
    assert ranges[0][0] == 0 and ranges[-1][1] == len(sizes) and ranges[0][1] == ranges[1][0]
    share = [sum(sizes[lo:hi]) for lo, hi in ranges]
    assert abs(share[0] - share[1]) <= max(sizes)  # balanced within one network
    expect = [k * 0.5 - 3.0 for k in range(len(sizes))]
    for r in range(world):
        assert np.allclose(res[r][2], expect)
        assert res[r][3] == 2.0  # max over ranks
        assert res[r][4] == float(sum(sizes))


def test_shard_single_rank():
    from itn_gb300 import distributed as D
    assert D.shard_networks([1, 2, 3], 0, 1) == (0, 3)
    assert D.max_over_ranks(3.5) == 3.5
