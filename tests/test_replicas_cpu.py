"""Replica runs of bench.py on several ranks (gloo, CPU): every rank times its
own replica, the ranks meet at a barrier, and the job's time is the maximum
over ranks.  There is no collective on the data path; these are the only
cross-rank calls the multi-GPU bench makes."""
import multiprocessing as mp
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank)})
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import bench
    r, w, local = bench.dist_info()
    dist.init_process_group("gloo", rank=r, world_size=w)
    bench.barrier(w)
    t = bench.max_over_ranks(10.0 + 5.0 * r, w)  # ms of this rank's timed region
    # the reference arm runs on rank 0 only; the other ranks return no line
    class A:
        workload, cases, steps, warmup = "ensemble", 1, 1, 1
    ref = bench.run_reference(A, r, w) if r != 0 else "rank0"
    bench.barrier(w)
    dist.destroy_process_group()
    out.put((r, w, local, t, ref))


@pytest.mark.timeout(600)
def test_two_ranks_barrier_and_max_time():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=540) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [x[0] for x in res] == [0, 1]
    for r, w, local, t, ref in res:
        assert w == 2 and local == r
        assert t == 15.0  # the slower rank's time is the job's time
    assert res[1][4] is None  # rank 1 runs no reference arm


def test_single_process_defaults(monkeypatch):
    sys.path.insert(0, ROOT)
    import bench
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    assert bench.dist_info() == (0, 1, 0)
    assert bench.max_over_ranks(3.5, 1) == 3.5
    bench.barrier(1)  # no process group: a no-op
