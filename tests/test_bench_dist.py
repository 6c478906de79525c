"""bench.py's multi-process path on CPU (gloo, world size 2): the slowest
rank's time is the job's, and the job's throughput counts every replica."""
import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    sys.path.insert(0, str(ROOT))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    w, r, _ = bench.dist_env()
    t = bench.max_over_ranks(1.0 + rank, dist)
    q.put((r, w, t, bench.job_throughput(w, 1000, 10, t)))
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_and_job_throughput_gloo():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[0] for o in out] == [0, 1]
    assert all(o[1] == 2 for o in out)
    assert all(o[2] == 2.0 for o in out)              # the slower rank's time
    assert all(abs(o[3] - 2 * 1000 * 10 / 2.0) < 1e-9 for o in out)


def test_reference_arm_other_ranks_exit_quietly(capsys, monkeypatch):
    sys.path.insert(0, str(ROOT))
    import bench
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")

    class A:
        workload, steps, warmup, gpus = "beam450", 1, 0, 2
    assert bench.run_reference(A()) is None
    assert capsys.readouterr().out == ""
