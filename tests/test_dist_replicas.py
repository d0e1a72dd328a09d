"""The multi-GPU paths of bench.py on CPU (gloo, world size 2): the
slowest-rank timing, the whole-job rate, the ensemble split, and the
reference arm's idle ranks.  No GPU: the same helpers run under NCCL on
GPU machines."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms = 10.0 + 5.0 * rank
    worst = bench.max_over_ranks(ms, dist, "cpu")
    ids = bench.shard(9, rank, world)
    gathered = [None] * world
    dist.all_gather_object(gathered, ids)
    out.put((rank, worst, gathered))
    dist.destroy_process_group()


def test_two_rank_timing_and_split():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, worst, gathered in res:
        assert worst == 15.0                      # the slowest rank's time, on every rank
        flat = sorted(i for part in gathered for i in part)
        assert flat == list(range(9))             # every scenario on exactly one rank


def test_whole_job_rate_and_single_rank():
    import bench
    assert bench.whole_job_rate(4, 1000, 2.0) == 2000.0
    assert bench.max_over_ranks(3.5, None, "cpu") == 3.5
    assert bench.shard(5, 0, 1) == [0, 1, 2, 3, 4]


def test_reference_arm_idle_on_other_ranks(monkeypatch, capsys):
    """Under torchrun only rank 0 times the reference; others exit 0 at once."""
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("LOCAL_RANK", "1")

    class A:
        n = 2048
        steps = 3
        warmup = 1
    assert bench.run_reference(A()) == 0
    assert capsys.readouterr().out == ""
