"""The multi-rank path of bench.py on the CPU: two gloo ranks, one process each.

The step is not sharded (one wall per GPU), so ranks are independent replicas;
what they share is the timing rule -- a barrier on both sides of the timed
region and the slowest rank's time -- and the reference arm's rule that rank 0
alone runs and prints while the other ranks exit 0 without work.
"""
import os
import socket
import sys

import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        bench.barrier(ws)
        slowest = bench.max_over_ranks(10.0 * (rank + 1), ws)
        bench.barrier(ws)
        assert bench.dist_env() == (ws, rank, rank)
        out.put((rank, slowest))
    finally:
        dist.destroy_process_group()


def test_two_replicas_take_the_slowest_time():
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    got = dict(out.get(timeout=5) for _ in range(2))
    assert got == {0: 20.0, 1: 20.0}


def test_reference_arm_runs_on_rank_0_only(monkeypatch, capsys):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("LOCAL_RANK", "1")
    assert bench.main(["--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "3"]) == 0
    assert capsys.readouterr().out == ""                       # no work and no line on the other ranks
