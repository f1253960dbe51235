"""Multi-GPU replicas: one process per GPU, MPC instances sharded across the
ranks with no data-path collective.  The instances are independent, so the
only exchanges are host-side: the max-over-ranks step time the benchmark
reports and, where a caller wants every result on one rank, a gather of the
per-instance result rows after the solves.
"""
import torch
import torch.distributed as dist


def shard(n_items, rank, world):
    """Contiguous [start, stop) share of n_items for `rank` (sizes differ by
    at most one)."""
    if world < 1 or not (0 <= rank < world):
        raise ValueError("bad rank/world")
    base, extra = divmod(int(n_items), int(world))
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def max_over_ranks(value, device=None):
    """Largest `value` over all ranks (step times: the job ends with its
    slowest rank).  Identity without an initialised process group."""
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def gather_rows(rows, n_items, device=None):
    """Every rank's result rows ([its shard, k] tensor, shard() order)
    assembled into one [n_items, k] CPU tensor on every rank."""
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return rows.detach().cpu()
    world = dist.get_world_size()
    k = rows.shape[1]
    longest = shard(n_items, 0, world)[1]
    pad = torch.zeros(longest, k, dtype=rows.dtype, device=device)
    pad[:rows.shape[0]] = rows.to(device)
    parts = [torch.empty_like(pad) for _ in range(world)]
    dist.all_gather(parts, pad)
    out = []
    for r in range(world):
        a, b = shard(n_items, r, world)
        out.append(parts[r][:b - a].cpu())
    return torch.cat(out, 0)
