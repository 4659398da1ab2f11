"""Batch sharding host logic with two gloo ranks on the CPU.

Each rank takes its shard, transforms it (here with the CPU oracle standing in
for the device: this test checks the sharding and gathering, not the
kernels), and the gathered result must equal the transform of the whole
batch; the timing reduction must return the slowest rank's time."""

import os
import socket

import numpy as np
import pytest
import torch
import torch.multiprocessing as mp

from adrt_gb300.dist import gather_shards, max_over_ranks, shard, shard_bounds


def test_shard_bounds_cover_batch():
    for batch in (0, 1, 5, 256, 257):
        for world in (1, 2, 3, 8):
            spans = [shard_bounds(batch, r, world) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == batch
            assert all(a[1] == b[0] for a, b in zip(spans, spans[1:]))
            sizes = [hi - lo for lo, hi in spans]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard_bounds(4, 2, 2)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, batch, q):
    import torch.distributed as dist

    from oracle import oracle

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        x = torch.from_numpy(np.random.default_rng(0).random((batch, 8, 8), dtype=np.float32))
        local = torch.from_numpy(oracle.adrt(shard(x, rank, world).numpy()))
        full = gather_shards(local, batch)
        t = max_over_ranks(float(rank + 1))
        if rank == 0:
            want = oracle.adrt(x.numpy())
            q.put((full.numpy().tobytes() == want.tobytes(), t))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("batch", [5, 8])
def test_two_rank_shard_and_gather(batch):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, batch, q)) for r in range(2)]
    for p in procs:
        p.start()
    ok, t = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert ok
    assert t == 2.0
