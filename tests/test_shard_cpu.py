"""Station sharding host logic, world size 2 on gloo (CPU)."""
import os
import socket

import numpy as np
import pytest

from ztm_gb300.shard import gather_slices, shard_range


def test_shard_range_partitions():
    for n in (0, 1, 7, 16384, 16385):
        for world in (1, 2, 3, 8):
            got = [shard_range(n, r, world) for r in range(world)]
            assert got[0][0] == 0 and got[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(got, got[1:]))
            assert max(h - l for l, h in got) - min(h - l for l, h in got) <= 1
    with pytest.raises(ValueError):
        shard_range(5, 2, 2)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, n, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    lo, hi = shard_range(n, rank, world)
    local = np.sin(np.arange(lo, hi) * 0.1)  # stands in for this rank's gz slice
    full = gather_slices(local, n)
    # max-over-ranks of the timed region, as the bench reduces it
    import torch
    t = torch.tensor([1.0 + rank])
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    q.put((rank, np.array_equal(full, np.sin(np.arange(n) * 0.1)), float(t.item())))
    dist.destroy_process_group()


@pytest.mark.parametrize("n", [16384, 1001])
def test_gather_of_disjoint_station_slices_two_ranks(n):
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, n, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert all(ok for _, ok, _ in res)
    assert all(t == 2.0 for _, _, t in res)
