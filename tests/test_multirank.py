"""Multi-rank host logic on CPU (gloo, world size 2): seed sharding covers
every seed exactly once, each rank gets its own beam, the timing is the max
over ranks."""
import os
import socket

import pytest


def test_shard_partition():
    from ufo_gb300.ranks import shard
    for n in (0, 1, 7, 512, 513):
        for world in (1, 2, 3, 8):
            spans = [shard(n, r, world) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(spans, spans[1:]))
            sizes = [b - a for a, b in spans]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard(10, 2, 2)


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR='127.0.0.1', MASTER_PORT=str(port))
    dist.init_process_group('gloo', rank=rank, world_size=world)
    from ufo_gb300.ranks import shard, max_over_ranks, beam_seed
    from ufo_gb300 import workloads as W
    lo, hi = shard(512, rank, world)
    beam = W.c2_beam(16, seed=beam_seed(rank))
    t = max_over_ranks(1.0 + rank)
    q.put((rank, lo, hi, float(beam[0, 0]), t))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks():
    import torch.multiprocessing as mp
    with socket.socket() as s:
        s.bind(('127.0.0.1', 0))
        port = s.getsockname()[1]
    ctx = mp.get_context('spawn')
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, lo0, hi0, b0, t0), (r1, lo1, hi1, b1, t1) = out
    assert (lo0, hi0, lo1, hi1) == (0, 256, 256, 512)
    assert b0 != b1          # independent beams per rank (weak scaling)
    assert t0 == t1 == 2.0   # the max over ranks
