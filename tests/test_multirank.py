"""Replica sharding across ranks, with world_size-2 gloo process groups on the CPU.

Events are independent, so N GPUs run N replicas; what needs checking is the host-side
bookkeeping: each rank's Philox window, the whole-channel shards of a batch, and the
max-over-ranks timing reduction.  Each rank computes its shard with the CPU oracle and the
shards are gathered (for the check only) and compared with one process doing everything."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from gpu_phs_gb300.replicas import channel_shards, event_window


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    import torch
    import torch.distributed as dist
    from gpu_phs_gb300 import processes as P
    from gpu_phs_gb300.philox import uniform_x
    from gpu_phs_gb300.replicas import channel_shards, event_window, max_over_ranks
    from oracle import oracle
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # 1. one process's event range split into per-rank Philox windows
        proc = P.tt()
        first, count = event_window(rank, world, 10001)
        x = uniform_x(42, count, proc.n_x, first_event=first)
        r = oracle.Oracle(proc, proc.sqrts).generate(x, threads=2)
        parts = [None] * world
        dist.all_gather_object(parts, (first, r.p, r.factor, r.ok))
        # 2. a multi-channel batch sharded by whole channels
        procs, counts = P.batched(seed=7, n_channels=12, total_events=6000)
        mine = channel_shards(counts, world)[rank]
        out = {}
        for c in mine:
            xc = uniform_x(100 + int(c), int(counts[c]), procs[c].n_x)
            out[int(c)] = oracle.Oracle(procs[c], 1000.0).generate(xc, threads=2).p
        shards = [None] * world
        dist.all_gather_object(shards, out)
        # 3. the slowest rank's time
        slowest = max_over_ranks(1.0 + rank)
        if rank == 0:
            q.put((parts, shards, slowest))
    finally:
        dist.destroy_process_group()


def test_event_windows_and_channel_shards_unit():
    for n, w in [(10, 3), (7, 7), (5, 8), (1 << 20, 4)]:
        spans = [event_window(r, w, n) for r in range(w)]
        assert spans[0][0] == 0 and sum(c for _, c in spans) == n
        assert all(spans[i][0] + spans[i][1] == spans[i + 1][0] for i in range(w - 1))
        assert max(c for _, c in spans) - min(c for _, c in spans) <= 1
    counts = np.array([500, 3, 90, 90, 1200, 7, 0, 64])
    sh = channel_shards(counts, 3)
    assert sorted(np.concatenate(sh).tolist()) == list(range(len(counts)))
    loads = [counts[s].sum() for s in sh]
    assert max(loads) - min(loads) <= counts.max()


def test_two_gloo_ranks_reproduce_one_process():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    try:
        # read before joining: rank 0's result is larger than a pipe buffer
        parts, shards, slowest = q.get(timeout=300)
    finally:
        for p in procs:
            p.join(timeout=60)
            if p.is_alive():
                p.kill()
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    assert slowest == 2.0

    from gpu_phs_gb300 import processes as P
    from gpu_phs_gb300.philox import uniform_x
    from oracle import oracle
    proc = P.tt()
    ref = oracle.Oracle(proc, proc.sqrts).generate(uniform_x(42, 10001, proc.n_x), threads=2)
    parts.sort(key=lambda t: t[0])
    assert np.array_equal(np.concatenate([t[1] for t in parts]), ref.p)
    assert np.array_equal(np.concatenate([t[2] for t in parts]), ref.factor)
    assert np.array_equal(np.concatenate([t[3] for t in parts]), ref.ok)

    procs_b, counts = P.batched(seed=7, n_channels=12, total_events=6000)
    merged = {}
    for d in shards:
        assert not set(d) & set(merged)          # every channel on one rank only
        merged.update(d)
    assert sorted(merged) == list(range(12))
    for c in range(12):
        xc = uniform_x(100 + c, int(counts[c]), procs_b[c].n_x)
        assert np.array_equal(merged[c], oracle.Oracle(procs_b[c], 1000.0).generate(xc, threads=2).p)
