"""The multi-GPU path of bench.py on CPU: two gloo ranks combine their time and work the way the
replicas do (max seconds, summed pairs), and the reference arm runs on rank 0 only."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        secs, pairs = bench.combine_ranks(1.0 + rank, 100.0 * (rank + 1), dist)
        dist.barrier()
        q.put((rank, secs, pairs))
    finally:
        dist.destroy_process_group()


def test_combine_ranks_two_gloo_ranks():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=180)
    for p in procs:
        if p.is_alive():
            p.kill()
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    got = sorted(q.get(timeout=10) for _ in procs)
    assert got == [(0, 2.0, 300.0), (1, 2.0, 300.0)]


def test_reference_arm_on_rank0_only(monkeypatch):
    sys.path.insert(0, ROOT)
    import bench
    calls = []
    monkeypatch.setattr(bench, "run_reference", lambda args: calls.append(args.impl))
    monkeypatch.setattr(sys, "argv", ["bench.py", "--impl", "reference", "--gpus", "2"])
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")
    bench.main()
    assert calls == []
    monkeypatch.setenv("RANK", "0")
    bench.main()
    assert calls == ["reference"]
