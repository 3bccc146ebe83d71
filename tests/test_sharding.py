"""One batch split over ranks (gcurval_gb300.sharding): contiguous curve
ranges balanced by the work estimate, and the gathered results of a
world-size-2 gloo job equal the one-rank results bit for bit.  The ranks'
compute is the oracle (CPU), so the test covers the split and the gather."""
import os
import socket

import numpy as np
import torch.distributed as dist
import torch.multiprocessing as mp

from gcurval_gb300 import datasets as ds
from gcurval_gb300 import sharding


def _batch():
    b = ds.uneven_batch(240, seed=4, max_ctrl=80, max_samples=40)
    b.sample_positions()
    return b


def _oracle_compute(sub):
    from oracle.oracle import Oracle
    o = Oracle(sub, nthreads=1)
    return o.lengths(), o.reverse(sub.n_samples, sub.positions, True, 0)


def test_ranges_are_contiguous_and_balanced():
    b = _batch()
    cost = ds.cost_proxy(b)
    for world in (1, 2, 3, 8):
        rs = sharding.shard_ranges(b, world)
        assert len(rs) == world and rs[0][0] == 0 and rs[-1][1] == b.n_curve
        assert all(r0[1] == r1[0] for r0, r1 in zip(rs, rs[1:]))
        assert all(hi > lo for lo, hi in rs)
        share = [cost[lo:hi].sum() for lo, hi in rs]
        # no rank is more than one curve's cost away from an even share
        assert max(share) - cost.sum() / world <= cost.max() + 1e-9
    # more ranks than curves: empty ranges at the end, nothing lost
    small = b.subset(np.arange(3))
    rs = sharding.shard_ranges(small, 5)
    assert sum(hi - lo for lo, hi in rs) == 3 and rs[-1][1] == 3


def _rank(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        L, u = sharding.sharded_run(_batch(), _oracle_compute, dist)
        out[rank] = (L, u)
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_ranks_reproduce_the_one_rank_results():
    b = _batch()
    L1, u1 = sharding.sharded_run(b, _oracle_compute, None)
    world = 2
    out = mp.Manager().dict()
    mp.spawn(_rank, args=(world, _free_port(), out), nprocs=world, join=True)
    for r in range(world):
        L, u = out[r]
        assert np.array_equal(L.view(np.uint64), L1.view(np.uint64))
        assert np.array_equal(u.view(np.uint64), u1.view(np.uint64))
