"""Multi-process host logic of the multi-GPU path, on CPU with gloo (world size 2)."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

from gisapr_gb300.replicas import job_rate, max_over_ranks, particle_shard, replica_seed, sum_over_ranks  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # per-rank step times: the job-wide rate uses the slowest rank
        times = max_over_ranks([1.0 + rank, 5.0 - rank, 0.25 * (rank + 1)])
        # particle shards: per-candidate partial scores add up to the full sums
        n = 11
        b, e = particle_shard(n, world, rank)
        per_particle = [[0.5 + 0.01 * i + c for i in range(n)] for c in range(3)]
        partial = [sum(row[b:e]) for row in per_particle]
        total = sum_over_ranks(partial)
        q.put((rank, times, (b, e), total, [sum(row) for row in per_particle], replica_seed(3, rank)))
    finally:
        dist.destroy_process_group()


def test_two_ranks_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = {}
    for _ in range(2):
        rank, *rest = q.get(timeout=120)
        out[rank] = rest
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank in (0, 1):
        times, shard, total, full, seed = out[rank]
        assert times == [2.0, 5.0, 0.5]
        for t, f in zip(total, full):
            assert abs(t - f) <= 1e-12 * abs(f)
    assert out[0][1] == (0, 6) and out[1][1] == (6, 11)
    assert out[0][4] != out[1][4]


def test_shards_cover_the_range_and_rate():
    for n in (0, 1, 7, 100, 5000):
        for world in (1, 2, 3, 8):
            ranges = [particle_shard(n, world, r) for r in range(world)]
            assert ranges[0][0] == 0 and ranges[-1][1] == n
            assert all(ranges[i][1] == ranges[i + 1][0] for i in range(world - 1))
            sizes = [e - b for b, e in ranges]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        particle_shard(10, 2, 2)
    assert job_rate(4, 10, 2.0) == 20.0
    assert max_over_ranks([1.5, 2.5]) == [1.5, 2.5]  # no process group: identity
