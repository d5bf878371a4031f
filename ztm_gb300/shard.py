"""Station sharding across ranks (one process per GPU).

Each station's gz is an independent sum over every prism, so a forward
shards by station with no exchange on the data path: every rank holds the
whole mesh and computes a contiguous slice of the stations; the only
collective is one gather of the disjoint slices when the caller wants the
full field on every rank.  (The reference has no distributed backend; its
parallelism is std::thread fan-out on one host, TFM.cpp:95-99.)"""
import numpy as np


def shard_range(n, rank, world):
    """Contiguous [lo, hi) slice of n items for rank (sizes differ by <= 1)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank/world")
    base, extra = divmod(n, world)
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def gather_slices(local, n, group=None):
    """All-gather disjoint contiguous slices (rank order) into the full
    length-n vector on every rank.  `local` is this rank's slice (numpy or
    torch); returns numpy float64."""
    import torch
    import torch.distributed as dist
    world = dist.get_world_size(group)
    sizes = [shard_range(n, r, world)[1] - shard_range(n, r, world)[0] for r in range(world)]
    width = max(sizes)
    t = torch.as_tensor(np.asarray(local, dtype=np.float64) if not torch.is_tensor(local)
                        else local.detach().to(torch.float64).cpu())
    pad = torch.zeros(width, dtype=torch.float64)
    pad[:t.numel()] = t
    outs = [torch.zeros(width, dtype=torch.float64) for _ in range(world)]
    dist.all_gather(outs, pad, group=group)
    return np.concatenate([o[:s].numpy() for o, s in zip(outs, sizes)])


def sharded_prism(ctx, mesh, rho, stations, rank, world, **kw):
    """This rank's slice of a prism forward: gz for stations[lo:hi]."""
    lo, hi = shard_range(len(stations), rank, world)
    return lo, hi, ctx.prism(mesh, rho, stations[lo:hi], **kw)
