"""Runs over several ranks (one process per GPU): replicas and agent shards.

The SB path exchanges nothing between agents, so ranks never talk while
they step.  Ranks either run independent replicas of a solve (weak scaling:
rank k uses seed + k) or disjoint agent ranges of one solve.  The only
collectives are on the host, after the run:

* the timing of a step: the maximum of the ranks' times and the sum of their
  work (all_reduce MAX / SUM);
* the statistics of the union of the ranks' agents, merged from per-rank
  summaries (count, min, max, mean, sum of squared deviations from the mean,
  agents at the maximum; merged pairwise as Chan, Golub and LeVeque's
  parallel variance, so no large sums of squares cancel) --
  the quantities src/ising.cu:238-265 reports (min, max, average, sample
  standard deviation, fraction of agents at the best cut).

Everything here runs on the host; with torch.distributed it works over gloo
(CPU) or NCCL alike.
"""
import math

import numpy as np


def agent_shard(agents, world, rank):
    """Contiguous agent range (offset, count) of rank out of world ranks;
    the first agents % world ranks take one agent more."""
    if world < 1 or not 0 <= rank < world or agents < 0:
        raise ValueError("bad shard request")
    base, extra = divmod(agents, world)
    off = rank * base + min(rank, extra)
    return off, base + (1 if rank < extra else 0)


SUMMARY_FIELDS = ("count", "min", "max", "mean", "m2", "n_at_max")


def local_summary(values):
    """Per-rank summary of agent values (cuts): count, min, max, mean, M2 (the
    sum of squared deviations from the rank's mean) and the number of agents
    at the maximum."""
    v = np.asarray(values, np.float64)
    if v.size == 0:
        return np.array([0.0, math.inf, -math.inf, 0.0, 0.0, 0.0])
    mx = float(v.max())
    mean = float(v.sum()) / v.size
    d = v - mean
    return np.array([float(v.size), float(v.min()), mx, mean, float(np.dot(d, d)),
                     float(np.count_nonzero(v == mx))])


def _chan(a, b):
    """(count, mean, M2) of the union of two parts (Chan, Golub, LeVeque)."""
    na, ma, m2a = a
    nb, mb, m2b = b
    if na == 0:
        return b
    if nb == 0:
        return a
    n = na + nb
    delta = mb - ma
    return n, ma + delta * (nb / n), m2a + m2b + delta * delta * (na * nb / n)


def merge_summaries(rows):
    """Statistics of the union from per-rank summaries: min, max, mean,
    sample standard deviation (denominator count - 1) and ps, the fraction of
    agents at the overall maximum.  Exact for min/max/ps; mean and std agree
    with the single-run values to rounding: the parts are merged pairwise
    (a balanced tree of Chan updates), never through a sum of squares."""
    rows = np.asarray(rows, np.float64).reshape(-1, len(SUMMARY_FIELDS))
    n = rows[:, 0].sum()
    if n == 0:
        raise ValueError("no agents")
    mx = rows[:, 2].max()
    at_max = rows[rows[:, 2] == mx, 5].sum()
    parts = [(r[0], r[3], r[4]) for r in rows]
    while len(parts) > 1:
        parts = [_chan(parts[i], parts[i + 1]) if i + 1 < len(parts) else parts[i]
                 for i in range(0, len(parts), 2)]
    _, mean, m2 = parts[0]
    std = math.sqrt(max(m2, 0.0) / (n - 1)) if n > 1 else math.nan
    return {"min": float(rows[:, 1].min()), "max": float(mx), "mean": float(mean), "std": std,
            "ps": float(at_max / n), "count": int(n)}


def reduce_timing(ms, units, device=None):
    """(max over ranks of ms, sum over ranks of units).  One process alone
    (no process group) returns its own numbers."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return float(ms), float(units)
    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    u = torch.tensor([float(units)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return float(t.item()), float(u.item())


def gather_statistics(values, device=None):
    """Statistics of all ranks' agent values, merged from per-rank summaries
    (one all_gather of six numbers per rank)."""
    import torch
    import torch.distributed as dist
    s = local_summary(values)
    if not (dist.is_available() and dist.is_initialized()):
        return merge_summaries([s])
    mine = torch.tensor(s, dtype=torch.float64, device=device)
    parts = [torch.empty_like(mine) for _ in range(dist.get_world_size())]
    dist.all_gather(parts, mine)
    return merge_summaries([p.cpu().numpy() for p in parts])
