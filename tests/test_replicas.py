"""Host side of runs over several ranks (no GPU): agent shards, the merge of
per-rank cut statistics, and the max/sum timing reduction -- over two gloo
ranks on the CPU, as bench.py uses them over NCCL."""
import os
import socket

import numpy as np
import pytest

import replicas


def _reference_stats(v):
    # src/ising.cu:238-265: min, max, average, sample std, fraction at max
    v = np.asarray(v, np.float64)
    return {"min": v.min(), "max": v.max(), "mean": v.mean(), "std": v.std(ddof=1),
            "ps": np.count_nonzero(v == v.max()) / v.size}


@pytest.mark.parametrize("agents,world", [(1024, 2), (1000, 3), (7, 8), (64, 1)])
def test_agent_shards_cover_every_agent_once(agents, world):
    seen = np.zeros(agents, np.int32)
    for rank in range(world):
        off, cnt = replicas.agent_shard(agents, world, rank)
        seen[off:off + cnt] += 1
    assert np.all(seen == 1)
    with pytest.raises(ValueError):
        replicas.agent_shard(agents, world, world)


def test_merged_statistics_equal_the_single_run():
    rng = np.random.default_rng(3)
    cuts = rng.integers(6900, 6960, size=1024).astype(np.float64)
    ref = _reference_stats(cuts)
    for world in (1, 2, 3, 5):
        parts = [replicas.local_summary(cuts[slice(*((o, o + c)))])
                 for o, c in (replicas.agent_shard(cuts.size, world, r) for r in range(world))]
        got = replicas.merge_summaries(parts)
        assert got["min"] == ref["min"] and got["max"] == ref["max"] and got["ps"] == ref["ps"]
        assert got["count"] == cuts.size
        assert abs(got["mean"] - ref["mean"]) <= 1e-12 * abs(ref["mean"])
        assert abs(got["std"] - ref["std"]) <= 1e-6 * ref["std"]
    # large cuts with a small spread (R-MAT scale: ~2.5e6 +- tens): a merge
    # through sums of squares cancels catastrophically, the pairwise one not
    big = 2.5e6 + rng.integers(0, 60, size=256).astype(np.float64)
    refb = _reference_stats(big)
    for world in (2, 3, 8):
        parts = [replicas.local_summary(big[o:o + c])
                 for o, c in (replicas.agent_shard(big.size, world, r) for r in range(world))]
        got = replicas.merge_summaries(parts)
        assert abs(got["std"] - refb["std"]) <= 1e-9 * refb["std"]
        assert abs(got["mean"] - refb["mean"]) <= 1e-15 * refb["mean"]
    # a rank with no agents changes nothing
    got = replicas.merge_summaries([replicas.local_summary(cuts), replicas.local_summary([])])
    assert got["max"] == ref["max"] and got["count"] == cuts.size


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, cuts, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        off, cnt = replicas.agent_shard(cuts.size, world, rank)
        stats = replicas.gather_statistics(cuts[off:off + cnt])
        ms, units = replicas.reduce_timing(10.0 + rank, 100 * (rank + 1))
        out.put((rank, stats, ms, units))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_merge_statistics_and_timing():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    rng = np.random.default_rng(5)
    cuts = rng.integers(100, 140, size=777).astype(np.float64)
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, cuts, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    ref = _reference_stats(cuts)
    for rank, stats, ms, units in res:
        assert ms == 11.0 and units == 300.0          # max of times, sum of work
        assert stats["max"] == ref["max"] and stats["min"] == ref["min"]
        assert stats["ps"] == ref["ps"] and stats["count"] == cuts.size
        assert abs(stats["std"] - ref["std"]) <= 1e-6 * ref["std"]
