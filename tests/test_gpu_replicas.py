"""Replica mode at the library level: two processes, each with its own copy of the library, map
and method, update their own particle filter on the GPU at the same time, and every rank's
weights equal the oracle's.  This is what `bench.py --gpus N` runs, one replica per rank with no
data exchange (weak scaling); the ranks meet only on the host (gloo) to agree on the outcome.
Both ranks use cuda:0 here (one GPU per run); their kernels never wait on each other.
"""
import os
import socket
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _replica(rank, world, port, out):
    for p in (ROOT, os.path.join(ROOT, "oracle")):
        if p not in sys.path:
            sys.path.insert(0, p)
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    import oracle as O
    import range_libc_gb300.range_libc as rl
    from range_libc_gb300 import workloads as W
    # each rank its own seeded filter (a replica of the same workload shape)
    wl = W.particle_filter_step(side=512, n_particles=400, n_beams=61, max_range_px=150.0, seed=300 + rank,
                                origin=(-2.0, 1.0))
    m = rl.PyOMap(np.ascontiguousarray(wl.occ.T))
    m.set_world(*wl.world[:4])
    g = rl.PyRayMarchingGPU(m, wl.max_range)
    g.set_sensor_model(wl.table)
    ref = O.OracleMethod(wl.occ, "rm", wl.max_range, world=m.world)
    ref.set_sensor_model(wl.table)
    _, trig = O.world_rays(m.world, wl.ins, wl.angles)
    g.set_trig_override(trig)
    dev = torch.device("cuda:0")
    ins, ang, obs = (torch.from_numpy(a).to(dev) for a in (wl.ins, wl.angles, wl.obs))
    w = torch.empty(len(wl.ins), dtype=torch.float64, device=dev)
    dist.barrier()
    for _ in range(20):   # both replicas keep the GPU busy at the same time
        g.calc_range_repeat_angles_eval_sensor_model(ins, ang, obs, w)
    torch.cuda.synchronize()
    dist.barrier()
    ok = np.array_equal(w.cpu().numpy(), ref.calc_range_repeat_angles_eval_sensor_model(wl.ins, wl.angles, wl.obs))
    flag = torch.tensor([1 if ok else 0], dtype=torch.int32)
    dist.all_reduce(flag, op=dist.ReduceOp.MIN)
    count = torch.tensor([len(wl.ins)], dtype=torch.int64)
    dist.all_reduce(count, op=dist.ReduceOp.SUM)
    out[rank] = (bool(ok), int(flag.item()), int(count.item()))
    dist.destroy_process_group()


def test_two_library_replicas_on_one_gpu():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")   # no fork of a process that may hold a CUDA context
    with ctx.Manager() as mgr:
        out = mgr.dict()
        procs = [ctx.Process(target=_replica, args=(r, world, port, out)) for r in range(world)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(300)
        assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
        assert dict(out) == {0: (True, 1, 800), 1: (True, 1, 800)}
