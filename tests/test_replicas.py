"""Multi-rank host logic on CPU (gloo, world size 2): instance partitioning
and the timing reduction the benchmark applies across replicas."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

from atmosphericturbulencesimul_gb300.replicas import aggregate, partition  # noqa: E402


def test_partition_covers_every_instance_once():
    for n in (0, 1, 7, 144, 145):
        for world in (1, 2, 3, 8):
            parts = [partition(n, r, world) for r in range(world)]
            seen = [i for p in parts for i in p]
            assert seen == list(range(n))
            sizes = [len(p) for p in parts]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        partition(4, 2, 2)


def test_aggregate_without_group():
    assert aggregate(2.0, 10) == (2.0, 10, 5.0)


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r ran 100 * (r + 1) frames in 1 + r seconds
        out[rank] = aggregate(1.0 + rank, 100 * (rank + 1))
        share = partition(144, rank, world)
        got = torch.tensor([len(share)], dtype=torch.int64)
        dist.all_reduce(got)
        out[rank + world] = int(got.item())
    finally:
        dist.destroy_process_group()


def test_aggregate_over_two_gloo_ranks():
    world = 2
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        port = _free_port()
        procs = [ctx.Process(target=_worker, args=(r, world, port, out)) for r in range(world)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        for r in range(world):
            t, n, v = out[r]
            assert t == 2.0 and n == 300 and v == 150.0     # slowest rank, all frames
            assert out[r + world] == 144                     # the shares cover the list
