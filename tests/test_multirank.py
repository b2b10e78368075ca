"""Multi-rank host logic on CPU: world_size-2 gloo process group.  Each rank
takes its particle shard (shard_range), evaluates and selects its shard with
the FP64 oracle standing in for that rank's GPU, the shards' lists are
all-gathered and merged (merge_accept_lists); the result must equal the
single-process acceptance over all particles, for eps and top-q modes."""
import os
import socket

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from abc_inference_transcription_gb300.host import local_select_q, merge_accept_lists, shard_range


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _problem():
    rng = np.random.default_rng(5)
    G, P, K = 12, 3001, 20
    base = np.abs(rng.normal(4.0, 2.0, (60, K))) + 0.2
    stats = base[rng.integers(0, 60, P)] * rng.lognormal(0, 0.25, (P, K))
    data = base[rng.integers(0, 60, G)]
    se = 0.1 * data * rng.lognormal(0, 0.5, (G, K))
    stats[10:20] = stats[9]  # ties across the shard boundary handled by index order
    return data, se, stats


def _worker(rank, world, port, mode, val, out_q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from oracle import oracle as orc
        data, se, stats = _problem()
        P = stats.shape[0]
        a, b = shard_range(P, rank, world)
        err = orc.errors(data, se, stats[a:b])
        q = local_select_q(val, P, b - a) if mode == 1 else val
        off, idx = orc.accept(err, mode, q)
        e = np.concatenate([err[idx[off[g]:off[g + 1]] - 1, g] for g in range(data.shape[0])])
        part = (off, idx + a, e)
        gathered = [None] * world
        dist.all_gather_object(gathered, part)
        if rank == 0:
            out_q.put(merge_accept_lists(gathered, mode, val, P))
        dist.barrier()
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("mode,val", [(0, 0.8), (1, 0.01), (1, 0.2)])
def test_two_rank_shards_merge_to_single_run(orc, mode, val):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, mode, val, q)) for r in range(2)]
    for p in procs:
        p.start()
    merged = q.get(timeout=120)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    data, se, stats = _problem()
    roff, ridx = orc.accept(orc.errors(data, se, stats), mode, val)
    assert np.array_equal(merged[0], roff)
    assert np.array_equal(merged[1], ridx)


def test_shard_range_partitions():
    for P in (0, 1, 7, 1000):
        for world in (1, 2, 3, 8):
            spans = [shard_range(P, r, world) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == P
            assert all(spans[i][1] == spans[i + 1][0] for i in range(world - 1))
