"""bench.py's multi-rank plumbing on CPU with gloo (world_size 2): every rank
runs a replica, the timed value is the maximum over ranks. The engine itself
does not shard (one GPU per replica, no collective on the data path)."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

from conftest import ROOT


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    import torch
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sys.path.insert(0, str(ROOT))
    t = torch.tensor([1.5 + rank], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.barrier()
    q.put((rank, float(t.item())))
    dist.destroy_process_group()


def test_max_over_ranks_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    assert got == [(0, 2.5), (1, 2.5)]


def test_bench_reference_arm_runs_on_rank0_only(monkeypatch, capsys):
    """--impl reference under N>1: ranks other than 0 exit without work."""
    sys.path.insert(0, str(ROOT))
    import bench

    class A:
        workload = "lle"
        steps = 1
        warmup = 1
        cpu_seconds = 0.1
        npts = None
        tmax = None
        precision = "fp32"

    called = []
    monkeypatch.setattr(bench, "cpu_sample_lle", lambda w, s: called.append(1) or {"value": 1.0, "unit": "x",
                                                                                 "cores": 1, "kind": "port",
                                                                                 "sample": "s"})
    bench.reference_arm(A(), 2, 1)
    assert not called and capsys.readouterr().out == ""
    bench.reference_arm(A(), 2, 0)
    assert called and '"impl": "reference"' in capsys.readouterr().out
