"""Two ranks over gloo (CPU): regions sharded with pilon_gb300.shard, each rank
computes its slice (with the oracle standing in for the per-GPU engine), and
rank 0 gathers the per-region results, which must equal a single-process run.
This exercises the host side of the multi-GPU path without a GPU."""
import os

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from pilon_gb300.shard import fold_insert_stats, shard_regions


def _work(rank, world, port, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from oracle import oracle
        from pilon_gb300 import _abi, synth
        from pilon_gb300.regions import plan_regions
        ds = synth.generate(3, scale=0.004)
        regs = plan_regions(ds.reads, [c.size for c in ds.contigs], chunk_size=6000)
        mine = shard_regions(regs, world)[rank]
        p = _abi.default_params()
        res = {}
        for i in mine:
            c, s, e, a, b = regs[i]
            r = oracle.process_region(ds.reads, p, ds.contigs[c], c, s, e, a, b)
            res[i] = (int(r.stats.base_count), int(r.stats.fr_count), int(r.stats.fr_sum), int(r.stats.fr_sumsq),
                      int(r.call.astype(np.int64).sum()), int(r.phys_cov.astype(np.int64).sum()))
        got = [None] * world
        dist.all_gather_object(got, res)
        if rank == 0:
            merged = {}
            for g in got:
                merged.update(g)
            q.put((len(regs), merged))
    finally:
        dist.destroy_process_group()


@pytest.mark.timeout(300)
def test_two_rank_sharding_matches_single_process():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_work, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    n, merged = q.get(timeout=240)
    for p in procs:
        p.join(60)
        assert p.exitcode == 0
    assert sorted(merged) == list(range(n))
    from oracle import oracle
    from pilon_gb300 import _abi, synth
    from pilon_gb300.regions import plan_regions
    ds = synth.generate(3, scale=0.004)
    regs = plan_regions(ds.reads, [c.size for c in ds.contigs], chunk_size=6000)
    stats = []
    for i, (c, s, e, a, b) in enumerate(regs):
        r = oracle.process_region(ds.reads, _abi.default_params(), ds.contigs[c], c, s, e, a, b)
        one = (int(r.stats.base_count), int(r.stats.fr_count), int(r.stats.fr_sum), int(r.stats.fr_sumsq),
               int(r.call.astype(np.int64).sum()), int(r.phys_cov.astype(np.int64).sum()))
        assert merged[i] == one
        stats.append(r.stats)
    run = fold_insert_stats(stats)
    assert run[-1][0] == sum(int(s.fr_count) for s in stats)


def test_shards_are_contiguous_and_balanced():
    regs = [(0, 1, 1000 * (k % 5 + 1)) for k in range(40)]
    sh = shard_regions(regs, 4)
    flat = [i for s in sh for i in s]
    assert flat == list(range(40))
    sizes = [sum(regs[i][2] for i in s) for s in sh]
    assert max(sizes) < 1.5 * min(sizes)
