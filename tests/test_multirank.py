"""The N > 1 path of bench.py on CPU: two gloo ranks set up the process
group, meet at the barrier, and agree on the max of their timings; the
reference arm runs on rank 0 only.  No GPU, no data-path collective (the
work shards into independent replicas)."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q, visible):
    import sys
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    if visible is None:
        os.environ.pop("CUDA_VISIBLE_DEVICES", None)
    else:
        os.environ["CUDA_VISIBLE_DEVICES"] = visible
    sys.path.insert(0, os.environ["GB300_REPO"])
    import bench
    r, w = bench.dist_setup()
    bench.barrier(w)
    m = bench.max_over_ranks(float(10 * (rank + 1)), w)
    # each rank pins itself to its own GPU index before any CUDA use
    q.put((r, w, m, os.environ.get("CUDA_VISIBLE_DEVICES")))
    import torch.distributed as dist
    dist.destroy_process_group()


@pytest.mark.parametrize("visible,expect", [(None, ["0", "1"]), ("4,5", ["4", "5"])])
def test_two_gloo_ranks_barrier_and_max(visible, expect):
    from conftest import REPO
    os.environ["GB300_REPO"] = REPO
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q, visible)) for r in range(2)]
    for p in procs:
        p.start()
    try:
        res = sorted(q.get(timeout=120) for _ in procs)
    finally:
        for p in procs:
            p.join(timeout=30)
            if p.is_alive():
                p.kill()
    assert all(p.exitcode == 0 for p in procs)
    assert [r[0] for r in res] == [0, 1]
    assert all(r[1] == 2 for r in res)
    assert all(r[2] == 20.0 for r in res)           # the max over both ranks
    assert [r[3] for r in res] == expect            # one GPU per rank


def _ref_worker(rank, world, port, q):
    import sys
    import io
    import contextlib
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, os.environ["GB300_REPO"])
    import bench

    class A:
        steps, warmup = 1, 3
    buf = io.StringIO()
    if rank == 0:
        bench.dist_setup()                 # joins the group; the CPU measurement itself is not run here
    else:
        with contextlib.redirect_stdout(buf):
            bench.run_reference(A())       # joins the group, then returns without work
    q.put((rank, buf.getvalue()))
    import torch.distributed as dist
    if dist.is_initialized():
        dist.destroy_process_group()


def test_reference_arm_rank_nonzero_exits_quietly():
    from conftest import REPO
    os.environ["GB300_REPO"] = REPO
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_ref_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    try:
        res = dict(q.get(timeout=120) for _ in procs)
    finally:
        for p in procs:
            p.join(timeout=30)
            if p.is_alive():
                p.kill()
    assert res[1] == ""                              # no line, no work on rank 1
