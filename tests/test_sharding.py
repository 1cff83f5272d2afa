"""Multi-rank host logic on CPU: world_size-2 gloo process groups on 127.0.0.1
(cell slices, maximum over ranks, the shared Courant step)."""
import os
import socket

import numpy as np
import pytest

from gpu_determ_gb300 import sharding


def test_shard_cells_partition():
    for total in (0, 1, 7, 4096, 4097):
        for world in (1, 2, 3, 8):
            slices = [sharding.shard_cells(total, world, r) for r in range(world)]
            assert sum(n for _, n in slices) == total
            assert slices[0][0] == 0
            for (a, n), (b, _) in zip(slices, slices[1:]):
                assert a + n == b
            assert max(n for _, n in slices) - min(n for _, n in slices) <= 1
    with pytest.raises(ValueError):
        sharding.shard_cells(10, 2, 2)


def test_single_process_fallbacks():
    assert sharding.max_over_ranks(3.5) == 3.5
    assert sharding.global_courant_dt(100.0, 0.5) == pytest.approx(0.005)


class _FakeDist:
    def __init__(self, backend):
        self.backend = backend

    def get_backend(self):
        return self.backend


def test_reduce_device_follows_backend(monkeypatch):
    torch = pytest.importorskip("torch")
    monkeypatch.setattr(torch.cuda, "current_device", lambda: 3)
    assert sharding.reduce_device(_FakeDist("nccl")) == torch.device("cuda", 3)   # NCCL reduces CUDA tensors
    assert sharding.reduce_device(_FakeDist("gloo")) == torch.device("cpu")
    assert sharding.reduce_device(None) == torch.device("cpu")
    assert sharding.reduce_device(_FakeDist("nccl"), device="cpu") == "cpu"      # the caller's choice wins


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import torch
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        first, count = sharding.shard_cells(4097, world, rank)
        # each rank's local maximum of nu' differs; the step must use the global one
        local_max = 50.0 + 30.0 * rank
        dt = sharding.global_courant_dt(torch.tensor([local_max]), 0.5)
        t = sharding.max_over_ranks(1.0 + rank)
        out.put((rank, first, count, dt, t))
    finally:
        dist.destroy_process_group()


def test_two_rank_gloo():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, f0, n0, dt0, t0), (r1, f1, n1, dt1, t1) = res
    assert (f0, n0) == (0, 2049) and (f1, n1) == (2049, 2048)
    expect = float(np.float32(0.5) / np.float32(80.0))
    assert dt0 == dt1 == pytest.approx(expect, rel=0, abs=0)
    assert t0 == t1 == 2.0
