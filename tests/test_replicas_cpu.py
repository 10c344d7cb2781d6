"""The multi-GPU mode of bench.py (independent replicas, one block per rank) on CPU ranks.

bench.py --gpus N runs one process per GPU; each rank solves its own block (seed + rank)
with no data-path collective, and the step time is the maximum over ranks.  These tests
run that host logic as two gloo ranks on the CPU: the max-over-ranks reduction, the
per-rank workloads and the reference arm's rank-0-only output.
"""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, ws, port, q):
    import sys

    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        import bench
        from psoci_gb300.inputs import named_workload

        w, r, loc = bench.dist_env()
        t = bench.barrier_max(1.5 + rank, w)  # each rank's step time; the job's is the slowest
        p = named_workload("fci_5e6o", seed=1 + r, ksym=1)
        q.put((r, w, loc, t, float(p.h[0, 0])))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_max_time_and_own_blocks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for pr in procs:
        pr.start()
    out = sorted(q.get(timeout=120) for _ in range(2))
    for pr in procs:
        pr.join(timeout=60)
        assert pr.exitcode == 0
    (r0, w0, l0, t0, h0), (r1, w1, l1, t1, h1) = out
    assert (r0, r1, w0, w1, l0, l1) == (0, 1, 2, 2, 0, 1)
    assert t0 == t1 == 2.5          # max over ranks, seen by every rank
    assert h0 != h1                 # seed + rank: each replica solves its own block


def test_reference_arm_prints_on_rank0_only(monkeypatch, capsys):
    import sys

    sys.path.insert(0, ROOT)
    import bench

    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")

    class Args:  # the arm returns before reading any argument on a rank other than 0
        pass

    bench.run_reference(Args())
    assert capsys.readouterr().out == ""
