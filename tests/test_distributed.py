"""The multi-GPU path on CPU: replicas (one per GPU under torchrun) split a library round robin and
report the whole job as the longest replica wall time and the summed work.  Two gloo ranks on
127.0.0.1 stand in for two GPUs; nothing here needs a device."""

import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, nsamples, queue):
    import os
    import torch.distributed as dist
    from holodeck_gb300.librarian import batch
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        idx = batch.shard_indices(nsamples, rank, world)
        local = dict(seconds=1.5 + rank, samples=len(idx), failed=rank, realizations=100 * len(idx),
                     draws=1.0e9 * len(idx), workers=3)
        queue.put((rank, idx, batch.reduce_stats(local)))
    finally:
        dist.destroy_process_group()


def test_library_shards_and_job_totals_with_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    queue = ctx.Queue()
    world, n = 2, 11
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, n, queue)) for r in range(world)]
    for p in procs:
        p.start()
    got = [queue.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    got.sort()
    shards = [g[1] for g in got]
    assert sorted(shards[0] + shards[1]) == list(range(n)) and not set(shards[0]) & set(shards[1])
    for _, _, job in got:   # every rank sees the same whole-job totals
        assert job["seconds"] == 2.5 and job["samples"] == n and job["failed"] == 1
        assert job["realizations"] == 100 * n and job["draws"] == 1.0e9 * n and job["ranks"] == world
        assert job["workers"] == 3


def test_shard_and_reduce_without_a_process_group():
    from holodeck_gb300.librarian import batch
    assert batch.shard_indices(5, 0, 1) == [0, 1, 2, 3, 4]
    assert batch.shard_indices(5, 1, 3) == [1, 4]
    with pytest.raises(ValueError):
        batch.shard_indices(5, 3, 3)
    st = dict(seconds=2.0, samples=3, failed=0, realizations=30, draws=5.0)
    assert batch.reduce_stats(st) == st
