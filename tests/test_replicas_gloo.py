"""The multi-GPU form is replicas only (no data-path collective): bench.py runs the same workload on
every rank and reduces the timings with a max over ranks.  This exercises that host-side logic
with two gloo ranks on the CPU: the max reduction, the barrier, the rendezvous on 127.0.0.1, and
the reference arm's rule that only rank 0 works and prints."""
import io
import os
import socket
import sys
from contextlib import redirect_stdout

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)
    import bench
    r, w = bench.dist_init(world)
    assert (r, w) == (rank, world)
    bench.barrier(w)
    m = bench.max_over_ranks(1.5 + rank, w)
    # the reference arm: ranks other than 0 return at once and print nothing
    buf = io.StringIO()
    if rank != 0:
        with redirect_stdout(buf):
            bench.run_reference_arm(bench.parse(["--impl", "reference", "--gpus", str(world)]), r, w)
    bench.barrier(w)
    out.put((rank, m, buf.getvalue()))
    import torch.distributed as dist
    dist.destroy_process_group()


def test_two_gloo_replicas_reduce_max_and_only_rank0_reports():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [m for _, m, _ in res] == [2.5, 2.5]
    assert res[1][2] == ""  # rank 1 printed nothing
