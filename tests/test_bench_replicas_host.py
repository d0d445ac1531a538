"""bench.py's replicas-only multi-GPU host logic on CPU (no GPU): two ranks
over gloo agree on the maximum step time and pass the barriers, and the
reference arm returns at once on ranks other than 0."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import bench
    r, w, local = bench.dist_setup(world)
    bench.barrier(w)
    step_s = 0.010 * (r + 1)  # rank 1 is the slower one
    worst = bench.allreduce_max(step_s, w)
    bench.barrier(w)
    ref = bench.run_reference(None, r, w, local) if r != 0 else "rank 0 runs it"
    import torch.distributed as dist
    dist.destroy_process_group()
    out.put((r, w, worst, ref))


def test_two_ranks_take_the_slowest_rank():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [g[0] for g in got] == [0, 1] and all(g[1] == 2 for g in got)
    assert all(g[2] == pytest.approx(0.020) for g in got)  # max over ranks
    assert got[1][3] is None  # the reference arm on rank 1: no work, no line


def test_single_rank_needs_no_process_group():
    import bench
    assert bench.allreduce_max(1.5, 1) == 1.5
    bench.barrier(1)
