"""bench.py's multi-process path on CPU: two gloo ranks, each a replica of the
workload (weak scaling), barrier around the timed region, max over ranks."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import bench
    r, ws, d = bench.dist_init()
    assert (r, ws) == (rank, world) and d is not None
    bench.barrier(d)
    # each rank reports its own elapsed time; the job time is the slowest rank's
    got = bench.max_over_ranks(d, 1.5 + rank)
    out[rank] = got
    d.destroy_process_group()


def test_two_gloo_ranks_take_the_max():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")   # no fork of a process that may hold a CUDA context
    with ctx.Manager() as mgr:
        out = mgr.dict()
        procs = [ctx.Process(target=_worker, args=(r, world, port, out)) for r in range(world)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
        assert all(p.exitcode == 0 for p in procs)
        assert dict(out) == {0: 2.5, 1: 2.5}
