"""The N>1 path of bench.py: replicas only.

Elements are independent, so N ranks run N independent replicas of the
workload (weak scaling) and meet only for the timing barrier and the max over
ranks; the reference arm runs on rank 0 alone.  These tests run two gloo ranks
on CPU."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, ws, port, out):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(ws), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)
    import bench
    w, r, local = bench.dist_init()
    bench.barrier(w)
    mx = bench.reduce_max(w, 1.5 + r)
    ds = bench.make_workload(8, seed=100 + r)          # each replica its own elements
    out.put((r, w, local, mx, ds.bases[:64].tobytes()))
    bench.barrier(w)
    import torch.distributed as td
    td.destroy_process_group()


def test_two_gloo_ranks_barrier_and_max():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [g[0] for g in got] == [0, 1]
    assert all(g[1] == 2 for g in got)
    assert all(g[3] == 2.5 for g in got)                # max over ranks reaches every rank
    assert got[0][4] != got[1][4]                        # replicas work on different elements


def test_reference_arm_runs_on_rank_zero_only(capsys):
    sys.path.insert(0, ROOT)
    import bench

    class Args:
        steps, warmup, gpus = 1, 0, 2

    bench.run_reference(Args(), 2, 1)                   # rank 1: returns at once, prints nothing
    assert capsys.readouterr().out == ""
