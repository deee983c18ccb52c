"""Multi-rank host logic of the replica path on CPU (gloo, world size 2)."""
import os
import socket

import pytest
import torch
import torch.multiprocessing as mp

from lime_gb300.replicas import shard_range


def test_shard_range_covers_every_instance_once():
    for n in (0, 1, 7, 4096):
        for world in (1, 2, 3, 8):
            seen = []
            for r in range(world):
                lo, hi = shard_range(n, r, world)
                assert 0 <= hi - lo <= n // world + 1
                seen.extend(range(lo, hi))
            assert seen == list(range(n))
    with pytest.raises(ValueError):
        shard_range(4, 2, 2)


def _free_port():
    s = socket.socket()
    s.bind(('127.0.0.1', 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import torch.distributed as dist
    from lime_gb300.replicas import shard_range, max_over_ranks, gather_to_rank0
    os.environ['MASTER_ADDR'] = '127.0.0.1'
    os.environ['MASTER_PORT'] = str(port)
    dist.init_process_group('gloo', rank=rank, world_size=world)
    try:
        lo, hi = shard_range(7, rank, world)
        local = torch.arange(lo, hi, dtype=torch.float64)[:, None] * torch.ones(1, 3)
        t = max_over_ranks(1.5 + rank)
        out = gather_to_rank0(local)
        q.put((rank, t, None if out is None else out.tolist()))
    finally:
        dist.destroy_process_group()


def test_gloo_two_ranks_timing_and_gather():
    ctx = mp.get_context('spawn')
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in range(2)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    res.sort()
    assert res[0][1] == res[1][1] == 2.5             # max over ranks
    assert res[1][2] is None
    assert [row[0] for row in res[0][2]] == list(range(7))
