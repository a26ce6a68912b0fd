"""World-size-2 gloo tests of the multi-GPU host logic on CPU: network sharding covers
every network exactly once with balanced work, max/sum over ranks, and the gather of
per-network log-norms (the only cross-rank exchange of the batched workload) -- with a real
BP solve of each rank's shard (the CPU oracle stands in for the rank's GPU) checked against
one solve of the whole batch."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "itensornetworksnext.jl_gb300")


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _batch(n_nets=9, seed=5):
    """Random 3-regular networks with uneven bonds and per-network seeded FP64 tensors (the
    tensors do not depend on how the batch is split)."""
    from itn_gb300 import graphs as G
    rng = np.random.default_rng(seed)
    nets, tens = [], []
    for k in range(n_nets):
        n = int(rng.integers(3, 9)) * 2
        edges = G.random_regular_edges(n, 3, rng)
        bonds = rng.choice([2, 3, 4], size=len(edges))
        g = G.from_edges(n, edges, bonds, phys=2)
        nets.append(g)
        tens.append(G.random_tensors(g, np.random.default_rng(1000 + k), np.float64, G.peps_scale(g)))
    return nets, tens


def _oracle_logz(g, t, sweeps):
    """Per-network Bethe log-norms of a batched graph after `sweeps` parallel sweeps (oracle)."""
    from oracle import oracle as O
    from itn_gb300 import graphs as G
    m, _, _, _ = O.bp_run(g, t, G.identity_messages(g), maxiter=sweeps)
    r = O.logscalars(g, t, m)
    und = np.flatnonzero(np.arange(g.nslots) < g.rev)
    src = np.repeat(np.arange(g.nv), np.diff(g.off))
    out = np.zeros(g.n_nets)
    np.add.at(out, g.net, r["logzv"][:, 0])
    np.add.at(out, g.net[src[und]], -r["logze"][:, 0])
    return out


def _worker(rank, world, port, sizes, out):
    import sys
    for p in (ROOT, PKG):
        sys.path.insert(0, p)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from itn_gb300 import distributed as D
        lo, hi = D.shard_networks(sizes, rank, world)
        t = D.max_over_ranks(1.0 + rank)
        work = D.sum_over_ranks(float(sum(sizes[lo:hi])))
        # a real solve of this rank's shard of a batch of networks
        nets, tens = _batch()
        blo, bhi, g = D.shard_batch(nets, rank, world)
        local = {}
        if g is not None:
            vals = _oracle_logz(g, np.concatenate(tens[blo:bhi]), 12)
            local = {blo + i: v for i, v in enumerate(vals)}
        logz = D.gather_logz(local, len(nets))
        out[rank] = (lo, hi, t, work, blo, bhi, logz.tolist())
    finally:
        dist.destroy_process_group()


def test_shard_solve_and_gather_world2():
    rng = np.random.default_rng(0)
    sizes = rng.integers(16, 257, size=37).tolist()
    world = 2
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    port = _free_port()
    mp.start_processes(_worker, args=(world, port, sizes, out), nprocs=world, join=True,
                       start_method="spawn")
    res = [out[r] for r in range(world)]
    ranges = [(r[0], r[1]) for r in res]
    assert ranges[0][0] == 0 and ranges[-1][1] == len(sizes) and ranges[0][1] == ranges[1][0]
    share = [sum(sizes[lo:hi]) for lo, hi in ranges]
    assert abs(share[0] - share[1]) <= max(sizes)  # balanced within one network
    for r in range(world):
        assert res[r][2] == 2.0  # max over ranks
        assert res[r][3] == float(sum(sizes))
    # every network solved on exactly one rank; the gathered log-norms equal one solve of the
    # whole batch
    nets, tens = _batch()
    assert res[0][4] == 0 and res[0][5] == res[1][4] and res[1][5] == len(nets) and res[0][5] > 0
    from itn_gb300 import graphs as G
    whole = _oracle_logz(G.batched(nets), np.concatenate(tens), 12)
    for r in range(world):
        np.testing.assert_allclose(res[r][6], whole, rtol=1e-12, atol=1e-12)


def test_shard_single_rank():
    from itn_gb300 import distributed as D
    assert D.shard_networks([1, 2, 3], 0, 1) == (0, 3)
    assert D.max_over_ranks(3.5) == 3.5
