#!/usr/bin/env python
"""Benchmark of the batched ray-casting path on GB300.

Default workload: one particle-filter update -- 4,000 particles x 61 beams
over 270 degrees on a seeded 2048x2048 corridor map at 0.05 m/px, ray
marching to 200 px, a 201x201 float64 sensor table -- through the fused
cast + sensor-model call (calc_range_repeat_angles_eval_sensor_model).

  value  rays/s with inputs resident in HBM, CUDA-event time of the fused
         kernel per step, L2 flushed (a 256 MiB write) before every step.
  e2e    the same call through the public Python API with host (pinned)
         numpy buffers, host<->device transfers inside the timed region: on
         Grace + Blackwell the kernel reads the poses, angles and
         observations from host memory and writes the weights back over
         NVLink-C2C (coherent host access); elsewhere they are copied.

Other workloads (--workload): plain (cast to ranges, then the separate
sensor model), batch (32 uneven filters in one persistent launch),
cddt (1M queries, td 108/216, 2048^2 map, --prune for PCDDT), glt
(GiantLUTCast build + 1M queries), radial (CDDT radial pairs), learned
(the MLP surrogate), published (the reference's own random / grid query
benchmark on its basement map, every method, its published figures beside).

--impl reference times the reference algorithm on the host cores instead
(the C restatement in oracle/, all threads).  Multi-GPU: every rank runs
its own replica of the workload (weak scaling); rank 0 reports.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "rays/s & particle updates/s, batched & learned vs plain GPU march, fixed error"


def load_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# ----------------------------------------------------------------- clocks
class ClockSampler:
    """SM clock and clock-event (throttle) reasons sampled during the timed region.

    Polls NVML (libnvidia-ml, read-only queries) every millisecond from a thread, so that even a
    few-millisecond timed region is sampled; falls back to `nvidia-smi -lms 200` without NVML.
    """

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    # nvmlClocksEventReason* bits (nvml.h)
    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown", 0x40: "hw_thermal_slowdown",
               0x80: "hw_power_brake_slowdown"}

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []
        self.t = None
        self.samples = []          # (sm_mhz, reason bits) from NVML
        self.max_mhz = None
        self.stop_flag = threading.Event()
        self.nvml = self._nvml_handle()

    def _nvml_handle(self):
        import ctypes as C
        try:
            L = C.CDLL("libnvidia-ml.so.1")
            if L.nvmlInit_v2() != 0:
                return None
            h = C.c_void_p()
            uuid = None
            try:   # the CUDA device's own UUID: NVML's index order can differ from CUDA's
                import torch
                uuid = "GPU-" + str(torch.cuda.get_device_properties(self.index).uuid)
            except (ImportError, AttributeError, RuntimeError, AssertionError):
                pass
            if uuid is None or L.nvmlDeviceGetHandleByUUID(uuid.encode(), C.byref(h)) != 0:
                if L.nvmlDeviceGetHandleByIndex_v2(C.c_uint(self.index), C.byref(h)) != 0:
                    return None
            mx = C.c_uint(0)
            if L.nvmlDeviceGetMaxClockInfo(h, C.c_int(1), C.byref(mx)) == 0:   # NVML_CLOCK_SM
                self.max_mhz = float(mx.value)
            reasons = getattr(L, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
                L.nvmlDeviceGetCurrentClocksThrottleReasons
            return L, h, reasons
        except (OSError, AttributeError):
            return None

    def _poll(self):
        import ctypes as C
        L, h, reasons = self.nvml
        mhz, bits = C.c_uint(0), C.c_ulonglong(0)
        while not self.stop_flag.is_set():
            if L.nvmlDeviceGetClockInfo(h, C.c_int(1), C.byref(mhz)) == 0 and reasons(h, C.byref(bits)) == 0:
                self.samples.append((float(mhz.value), int(bits.value)))
            time.sleep(0.001)

    def start(self):
        if self.nvml is not None:
            self.t = threading.Thread(target=self._poll, daemon=True)
            self.t.start()
            while not self.samples and self.t.is_alive():   # sampling before the region starts
                time.sleep(0.0005)
            return
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.t = threading.Thread(target=self._read, daemon=True)
        self.t.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.nvml is not None:
            self.stop_flag.set()
            if self.t:
                self.t.join(timeout=2)
            sm = [m for m, _ in self.samples]
            reasons = sorted({n for _, b in self.samples for bit, n in self.REASONS.items() if b & bit})
            return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": self.max_mhz,
                    "reasons": reasons, "samples": len(sm), "source": "nvml, 1 ms polling"}
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.t:
            self.t.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm), "source": "nvidia-smi -lms 200"}


# ----------------------------------------------------------------- distributed
_DIST = None


def dist_init():
    """(rank, world size, torch.distributed or None); the process group is set up once."""
    global _DIST
    if _DIST is None:
        _DIST = _dist_setup()
    return _DIST


def _dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws <= 1:
        return 0, 1, None
    import torch
    import torch.distributed as dist
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    backend = "nccl" if torch.cuda.is_available() else "gloo"
    if torch.cuda.is_available():
        torch.cuda.set_device(local)
    dist.init_process_group(backend=backend)
    return rank, ws, dist


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, v: float) -> float:
    if dist is None:
        return v
    import torch
    dev = torch.device("cuda", torch.cuda.current_device()) if torch.cuda.is_available() else torch.device("cpu")
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ----------------------------------------------------------------- workloads
def build_pf(rl, W, args):
    wl = W.particle_filter_step()
    omap = rl.PyOMap(np.ascontiguousarray(wl.occ.T))
    omap.set_world(*wl.world[:4])
    method = rl.PyRayMarchingGPU(omap, wl.max_range)
    method.set_sensor_model(wl.table)
    return wl, omap, method


SHIPPED_BUILD = ("oracle/ C restatement built with the reference's shipped flags (-O3 -ffast-math "
                 "-fno-math-errno, -march=native spelled -mcpu=neoverse-v2 on Grace)")


def cpu_reference_pf(wl, world, steps, warmup, budget_s, nthreads, fast=True):
    """The reference algorithm (C restatement, oracle/) on the host cores: full
    particle-filter steps until `budget_s` seconds or `steps` steps.  fast: the build with the
    reference's shipped optimisation flags (the speed baseline); else the strict parity build."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    O.build(reference=False)
    ref = O.OracleMethod(wl.occ, "rm", wl.max_range, world=world, fast=fast)
    ref.set_sensor_model(wl.table)
    for _ in range(max(warmup, 0)):
        ref.calc_range_repeat_angles_eval_sensor_model(wl.ins, wl.angles, wl.obs, nthreads=nthreads)
    done, t0 = 0, time.perf_counter()
    while True:
        ref.calc_range_repeat_angles_eval_sensor_model(wl.ins, wl.angles, wl.obs, nthreads=nthreads)
        done += 1
        el = time.perf_counter() - t0
        if done >= steps or el >= budget_s:
            break
    rays = done * len(wl.ins) * len(wl.angles)
    return rays / el, done, el


def pf_config(kind: str, n: int, na: int) -> dict:
    """The `config` of the particle-filter lines (both arms)."""
    return {"workload": f"particle-filter step ({kind}): corridor 2048^2 @0.05 m/px, "
                        f"{n} particles x {na} beams over 270 deg, RM max_range 200 px, 201x201 f64 sensor table",
            "particles": n, "beams": na, "map": "2048x2048 corridor, seed 2000"}


def run_reference(args):
    """--impl reference: the reference's CPU implementation on the host cores (all threads; one
    thread reported beside it)."""
    from range_libc_gb300 import workloads as W
    rank, ws, dist = dist_init()
    if rank != 0:
        return 0
    wl = W.particle_filter_step()
    world = tuple(float(np.float32(v)) for v in (wl.world[0], wl.world[1], wl.world[2], wl.world[3], 0.0, 1.0))
    nthreads = os.cpu_count() or 1
    val, done, el = cpu_reference_pf(wl, world, args.steps, args.warmup, budget_s=60.0, nthreads=nthreads)
    v1, d1, e1 = cpu_reference_pf(wl, world, 1000, 1, budget_s=5.0, nthreads=1)
    vs, ds, es = cpu_reference_pf(wl, world, 1000, 1, budget_s=5.0, nthreads=nthreads, fast=False)
    n, na = len(wl.ins), len(wl.angles)
    line = {
        "impl": "reference", "metric": METRIC, "value": val, "unit": "rays/s", "n_gpus": ws,
        "gpus_used": 0, "devices": "host CPU cores of rank 0 (the reference's path has no GPU code here)",
        "steps": done, "warmup": args.warmup, "ms_per_step": 1e3 * el / done, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 ranges / f64 weights", "data": "synthetic",
        "config": dict(pf_config(args.workload if args.workload in ("fused", "plain") else "fused", n, na),
                       l2="no device cache to flush: host CPU run"),
        "particle_updates_per_s": val / na,
        "cpu_baseline": {"value": val, "unit": "rays/s", "cores": nthreads, "kind": "port",
                         "build": "shipped flags",
                         "sample": f"{done} full steps ({n}x{na} rays each), {SHIPPED_BUILD}, {nthreads} threads",
                         "single_thread": {"value": v1, "sample": f"{d1} full steps in {e1:.1f} s, 1 thread"},
                         "strict_build": {"value": vs, "sample": f"{ds} full steps in {es:.1f} s, the parity build "
                                                                 f"(-O3 -ffp-contract=off), {nthreads} threads"}},
        "e2e": {"value": val, "unit": "rays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


# DRAM bytes (read + write) per launch of the dominant kernel, from one `ncu --set full` capture
# of the same workload (the k_fused and k_batch summaries under profiles/)
# per distance-transform layout of the fused kernel (the schedules the autotuner picks here)
FUSED_NCU_TRAFFIC = {
    0: (512_256, "ncu dram__bytes_read.sum + dram__bytes_write.sum, k_fused<RM, linear DT>, this workload "
                 "(the kernel version with 16-bit range bins in shared memory)"),
    4: (522_112, "ncu dram__bytes_read.sum + dram__bytes_write.sum, k_fused<RM, step map>, this workload "
                 "(mean of 2 launches: 521,984 and 522,240 B read, 0 written; the kernel version with 16-bit "
                 "range bins in shared memory)"),
    5: (566_400, "ncu dram__bytes_read.sum + dram__bytes_write.sum, k_fused<RM, step map with equal-step runs>, "
                 "this workload (mean of 2 launches: 566,528 and 566,272 B read, 0 written)"),
}
BATCH_NCU_TRAFFIC = {
    6: (501_862_656 + 35_385_856, "ncu dram__bytes_read.sum + dram__bytes_write.sum of k_batch on the first 6 "
                                   "filters (--filters 6), schedule step map / 256 threads / 8 particles per tile / "
                                   "separate products"),
    32: (2_628_463_616 + 402_988_544, "ncu dram__bytes_read.sum + dram__bytes_write.sum of k_batch, all 32 filters, "
                                      "schedule step map / 256 threads / 8 particles per tile / separate products"),
}


# The reference's published single-call figures (Jetson TX1; CPU methods on one thread, RMGPU on
# its GPU) for its own benchmark: maps/basement_hallways_5cm.png, max_range 500, theta_disc 108,
# queries per second of Benchmark::random_sample and grid_sample.
PUBLISHED_TX1 = {"bl": (297e3, 360e3), "rm": (1.17e6, 1.6e6), "rmgpu": (18e6, 28e6), "cddt": (2.09e6, 4.25e6),
                 "pcddt": (2.26e6, 4.47e6), "glt": (2.16e6, 4.85e6)}


def run_published(args):
    """The reference's own benchmark on its own map, with the published figures beside ours:
    basement_hallways_5cm (1200^2, the reference's PNG loaded by its own loader, kept as a golden
    fixture), max_range 500 px, theta_discretization 108; `random`: queries x ~ U[1, W-1),
    y ~ U[1, H-1), theta ~ U[0, 2 pi) (Benchmark::random_sample, 10x its 200,000 queries per step);
    `grid`: every 10 px in x and y at 40 angles i * 2 pi / 40 (Benchmark::get_grid_samples,
    576,000 queries).  calc_range in the grid frame (no world transform), device-resident queries,
    CUDA events per call, L2 flushed before each."""
    import torch
    import range_libc_gb300.range_libc as rl
    from range_libc_gb300 import _lib

    rank, ws, dist = dist_init()
    dev = torch.device("cuda", torch.cuda.current_device())
    stream = torch.cuda.current_stream(dev)
    gold = np.load(os.path.join(ROOT, "tests", "golden", "reference_vectors.npz"))
    occ = gold["basement/occ"]
    W_, H_ = occ.shape
    omap = rl.PyOMap(np.ascontiguousarray(occ.T))
    rng = np.random.default_rng(1903)
    n_rand = 2_000_000
    qr = np.stack([rng.uniform(1.0, W_ - 1.0, n_rand), rng.uniform(1.0, H_ - 1.0, n_rand),
                   rng.uniform(0.0, 6.28318530718, n_rand)], 1).astype(np.float32)
    coeff = np.float32(2.0 * math.pi / 40)
    gx, gy = np.meshgrid(np.arange(0, W_, 10), np.arange(0, H_, 10), indexing="ij")
    qg = np.concatenate([np.stack([gx.ravel(), gy.ravel(), np.full(gx.size, np.float32(i) * coeff)], 1)
                         for i in range(40)]).astype(np.float32)
    t0 = time.perf_counter()
    methods = {"bl": rl.PyBresenhamsLine(omap, 500.0), "rm": rl.PyRayMarchingGPU(omap, 500.0),
               "cddt": rl.PyCDDTCast(omap, 500.0, 108)}
    pc = rl.PyCDDTCast(omap, 500.0, 108)
    pc.prune()
    methods["pcddt"] = pc
    methods["glt"] = rl.PyGiantLUTCast(omap, 500.0, 108)
    torch.cuda.synchronize()
    setup_s = time.perf_counter() - t0
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    dq = {"random": torch.from_numpy(qr).to(dev), "grid": torch.from_numpy(qg).to(dev)}
    outs = {k: torch.empty(len(v), dtype=torch.float32, device=dev) for k, v in dq.items()}
    res, launches = {}, 0
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    for name, m in methods.items():
        res[name] = {}
        for bench_name, q in dq.items():
            o = outs[bench_name]
            best = None
            for search in ((0, 2) if name in ("cddt", "pcddt") else (0,)):   # CDDT: binary / sector search
                if name in ("cddt", "pcddt"):
                    m.set_schedule(0, 0, search, 0)

                def step():
                    _lib.call("rlc_calc_range_many", m.handle, C_vp(q.data_ptr()), C_vp(o.data_ptr()), len(q),
                              _lib.RLC_NO_WORLD | _lib.RLC_DEVICE_PTRS, C_vp(stream.cuda_stream))
                    return 1
                for _ in range(args.warmup):
                    step()
                t, nl = _event_steps(torch, stream, args.steps, flush, step)
                launches += nl
                rate = len(q) * args.steps / (sum(t) / 1e3)
                best = rate if best is None else max(best, rate)
            pub = PUBLISHED_TX1["rmgpu" if name == "rm" else name][0 if bench_name == "random" else 1]
            res[name][bench_name] = {"queries_per_s": best, "published_tx1": pub, "ratio": best / pub}
    clk = clocks.stop()
    if rank != 0:
        return 0
    cpu = None
    if not args.no_cpu_baseline:   # the oracle (C restatement of the reference) on one host thread
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as O
        O.build(reference=False)
        cpu = {}
        sample = qr[:100_000]
        for name in ("bl", "rm", "cddt", "pcddt"):
            om = O.OracleMethod(occ, name, 500.0, td=108, nthreads=os.cpu_count() or 1)
            t0 = time.perf_counter()
            om.calc_range_many_raw(sample, nthreads=1)
            cpu[name] = len(sample) / (time.perf_counter() - t0)
    value = res["rm"]["random"]["queries_per_s"] * ws
    line = {
        "metric": "queries/s of the reference's random_sample benchmark (RM; every method beside it)", "value": value,
        "unit": "queries/s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": value / PUBLISHED_TX1["rmgpu"][0], "dtype": "f32", "data": "the reference's map",
        "config": {"workload": "reference benchmark: basement_hallways_5cm 1200^2, max_range 500, theta_disc 108, "
                               f"random {n_rand} / grid {len(qg)} queries per call",
                   "l2": "flushed before every call (256 MiB write)",
                   "baseline": "published Jetson TX1 figures (RMGPU on its GPU, CPU methods on one thread)"},
        "methods": res, "setup_s": setup_s, "gpu_launches": launches, "clocks": clk,
        "cpu_baseline": None if cpu is None else {
            "value": cpu["rm"], "unit": "queries/s", "cores": 1, "kind": "port",
            "sample": "100,000 of the random queries, oracle/ C restatement, one thread, per method",
            "methods": cpu},
    }
    print(json.dumps(line))
    return 0


def C_vp(v):
    import ctypes
    return ctypes.c_void_p(v)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="fused",
                    choices=["fused", "plain", "batch", "cddt", "learned", "glt", "radial", "published"])
    ap.add_argument("--train-rays", type=int, default=64_000_000, help="learned workload: training rays")
    ap.add_argument("--train-batch", type=int, default=8192, help="learned workload: rays per training step")
    ap.add_argument("--train-lr", type=float, default=2e-3, help="learned workload: Adam learning rate")
    ap.add_argument("--td", type=int, default=108, help="cddt workload: theta discretization")
    ap.add_argument("--prune", action="store_true", help="cddt workload: pruned table (PCDDT)")
    ap.add_argument("--filters", type=int, default=32, help="batch workload: number of filters")
    ap.add_argument("--no-plain", action="store_true", help="batch workload: skip the per-call comparisons")
    ap.add_argument("--oracle-check", action="store_true", help="batch workload: check the weights against the oracle")
    ap.add_argument("--fused-only", action="store_true",
                    help="fused workload: skip the batched and learned figures added to its line")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--schedule", default=None,
                    help="fixed schedule instead of the autotuner (for profiling): fused 'layout,block,prefetch,tile', "
                         "batch 'layout,prefetch,block,tile[,separate products 0/1]'")
    ap.add_argument("--out", default=None, help="also write the JSON line to this file")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "batch":
        run_batch(args, oracle_check=args.oracle_check)
        return 0
    if args.workload == "cddt":
        return run_cddt(args)
    if args.workload == "learned":
        run_learned(args)
        return 0
    if args.workload == "glt":
        return run_glt(args)
    if args.workload == "radial":
        return run_radial(args)
    if args.workload == "published":
        return run_published(args)

    import torch
    import range_libc_gb300.range_libc as rl
    from range_libc_gb300 import workloads as W

    rank, ws, dist = dist_init()
    dev_index = torch.cuda.current_device()
    dev = torch.device("cuda", dev_index)
    stream = torch.cuda.current_stream(dev)

    wl, omap, method = build_pf(rl, W, args)
    n, na = len(wl.ins), len(wl.angles)
    rays_per_step = n * na
    ins = torch.from_numpy(wl.ins).to(dev)
    angles = torch.from_numpy(wl.angles).to(dev)
    obs = torch.from_numpy(wl.obs).to(dev)
    weights = torch.empty(n, dtype=torch.float64, device=dev)
    ranges = torch.empty(rays_per_step, dtype=torch.float32, device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def step():
        if args.workload == "fused":
            method.calc_range_repeat_angles_eval_sensor_model(ins, angles, obs, weights)
            return 1
        method.calc_range_repeat_angles(ins, angles, ranges)
        method.eval_sensor_model(obs, ranges, weights, na, n)
        return 2

    # autotune the schedule on this workload (or take the given one), then warm up
    tune_table = None
    if args.workload == "fused":
        if args.schedule:
            method.set_schedule(*[int(v) for v in args.schedule.split(",")])
        else:
            # the timed steps run after an L2 flush, so the candidates are timed the same way
            method.autotune(ins, angles, obs, weights, flush_l2=True)
            res = sorted(method.autotune_results(), key=lambda r: r[2] if r[2] is not None else 1e9 + r[1])
            tune_table = [{"schedule": list(sc), "median_ms": round(m1, 5),
                           "final_median_ms": None if m2 is None else round(m2, 5)} for sc, m1, m2 in res[:6]]
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()

    # ---- device-resident timing: CUDA events around each step, L2 flushed before it
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    clocks = ClockSampler(dev_index)
    launches = 0
    gpu_lead_in(torch, 0.0)               # loads the spin kernel before the timed region
    barrier(dist)
    torch.cuda.synchronize()
    clocks.start()
    gpu_lead_in(torch)
    for u in range(UNTIMED_AFTER_LEAD_IN):   # untimed: the first steps after the lead-in
        flush.fill_(-1.0 - u)
        step()
    for k in range(args.steps):
        flush.fill_(float(k + 1))
        starts[k].record(stream)
        launches += step()
        ends[k].record(stream)
    torch.cuda.synchronize()
    barrier(dist)
    clk = clocks.stop()
    per_step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    total_ms = max_over_ranks(dist, sum(per_step_ms))
    value = ws * rays_per_step * args.steps / (total_ms / 1e3)

    # ---- end to end through the public API with pinned host buffers
    h_ins = torch.from_numpy(wl.ins).pin_memory().numpy()
    h_ang = torch.from_numpy(wl.angles).pin_memory().numpy()
    h_obs = torch.from_numpy(wl.obs).pin_memory().numpy()
    h_w = torch.empty(n, dtype=torch.float64).pin_memory().numpy()
    h_r = torch.empty(rays_per_step, dtype=torch.float32).pin_memory().numpy()

    def step_host():
        if args.workload == "fused":
            method.calc_range_repeat_angles_eval_sensor_model(h_ins, h_ang, h_obs, h_w)
        else:
            method.calc_range_repeat_angles(h_ins, h_ang, h_r)
            method.eval_sensor_model(h_obs, h_r, h_w, na, n)

    for _ in range(args.warmup):
        step_host()
    e2e_s = 0.0
    barrier(dist)
    for k in range(args.steps):
        flush.fill_(float(k))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        step_host()                       # synchronous: results are in h_w on return
        e2e_s += time.perf_counter() - t0
    barrier(dist)
    e2e_s = max_over_ranks(dist, e2e_s)
    e2e = ws * rays_per_step * args.steps / e2e_s
    h2d = wl.ins.nbytes + wl.angles.nbytes + wl.obs.nbytes
    d2h = n * 8
    if args.workload == "plain":
        h2d += wl.obs.nbytes + rays_per_step * 4
        d2h += rays_per_step * 4

    # correctness check of the timed configuration against the host path
    torch.cuda.synchronize()
    dev_w = weights.cpu().numpy()
    if not np.array_equal(dev_w, h_w):
        raise SystemExit("bench: device and host paths disagree")

    # ---- roofline of the dominant kernel (the fused cast + sensor model)
    total_steps = method.count_steps(wl.ins, wl.angles)
    # per particle 12 B pose + 8 B weight; per ray one 8 B table read + 4 B per distance-transform read
    alg_bytes = n * (12 + 8) + rays_per_step * 8 + 4 * total_steps
    kern_s = (sum(per_step_ms) / args.steps) / 1e3
    peak, peak_kind = load_peaks()
    achieved = alg_bytes / kern_s / 1e9
    traffic, traffic_src = FUSED_NCU_TRAFFIC.get(method.schedule()[0], (None, "no capture of this layout"))
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": traffic, "traffic_source": traffic_src,
                "peak_source": f"hbm_gbs burst ({peak_kind})",
                "algorithmic_bytes_per_launch": alg_bytes, "mean_march_steps_per_ray": total_steps / rays_per_step,
                "kernel": "k_fused (cast + sensor model)"}

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        nthreads = os.cpu_count() or 1
        v1, d1, e1 = cpu_reference_pf(wl, omap.world, steps=100000, warmup=1, budget_s=10.0, nthreads=nthreads)
        s1, sd, se = cpu_reference_pf(wl, omap.world, steps=100000, warmup=1, budget_s=3.0, nthreads=1)
        vs, ds, es = cpu_reference_pf(wl, omap.world, steps=100000, warmup=1, budget_s=3.0, nthreads=nthreads,
                                      fast=False)
        cpu = {"value": v1, "unit": "rays/s", "cores": nthreads, "kind": "port", "build": "shipped flags",
               "sample": f"{d1} full steps ({n}x{na} rays each) in {e1:.1f} s, {SHIPPED_BUILD}, {nthreads} threads",
               "single_thread": {"value": s1, "sample": f"{sd} full steps in {se:.1f} s, 1 thread"},
               "strict_build": {"value": vs, "sample": f"{ds} full steps in {es:.1f} s, the parity build "
                                                       f"(-O3 -ffp-contract=off), {nthreads} threads"}}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "rays/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 ranges / f64 weights", "data": "synthetic",
            "config": dict(pf_config(args.workload, n, na), l2="flushed before every step (256 MiB write)"),
            "schedule": dict(zip(("dt_layout", "block", "prefetch", "tile"), method.schedule()),
                             autotune_candidates=tune_table,
                             autotune="median of 5 launches per candidate, then of 31 for the best 3, "
                                      "L2 flushed before each"),
            "particle_updates_per_s": value / na,
            "step_us": {"min": 1e3 * min(per_step_ms), "median": 1e3 * statistics.median(per_step_ms),
                        "max": 1e3 * max(per_step_ms), "max_at_step": per_step_ms.index(max(per_step_ms))},
            "e2e": {"value": e2e, "unit": "rays/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "particle_updates_per_s": e2e / na},
            "gpu_launches": launches,
            "roofline": roofline,
            "cpu_baseline": cpu,
            "clocks": clk,
        }
    if args.workload == "fused" and not args.fused_only:
        line_bl = batched_and_learned_figures(args, value)
        if rank == 0:
            line["batched_and_learned"] = line_bl
    if rank == 0:
        s = json.dumps(line)
        print(s)
        if args.out:
            with open(args.out, "w") as f:
                f.write(s + "\n")
    if dist is not None:
        dist.destroy_process_group()
    return 0


def batched_and_learned_figures(args, fused_value):
    """The ratios the metric names, measured in the same run as the particle-filter step: the
    32-filter batch against plain per-call GPU casts (weights checked against the oracle), and the
    learned surrogate against the exact path."""
    out = {}
    b = run_batch(args, emit=False, oracle_check=True)
    out["batched"] = {k: b.get(k) for k in (
        "value", "unit", "ms_per_step", "particle_updates_per_s", "plain_per_call_rays_per_s",
        "per_filter_fused_rays_per_s", "batched_over_plain", "weights_equal_plain", "weights_vs_oracle",
        "roofline", "clocks", "gpu_launches")}
    out["batched"]["config"] = b.get("config")
    ln = run_learned(args, emit=False)
    out["learned"] = {k: ln.get(k) for k in (
        "value", "unit", "ms_per_step", "exact_repeat_angles_rays_per_s", "exact_fused_rays_per_s",
        "learned_over_exact", "fallback_rate", "heldout_t_error_px", "range_error_px_all",
        "range_error_px_accepted", "weight_error")}
    out["learned"]["config"] = ln.get("config")
    out["learned"]["learned_over_batched_exact"] = ln["value"] / b["value"] if b.get("value") else None
    out["batched_over_particle_filter_step"] = b["value"] / fused_value if fused_value else None
    return out


_LEAD_IN_READY = False


UNTIMED_AFTER_LEAD_IN = 3


def gpu_lead_in(torch, ms: float = 2.0):
    """Queue ~`ms` of GPU work (a spin kernel) ahead of a timed loop, so that the host has queued
    the loop's first steps before the GPU reaches them: a host-side pause (the clock sampler's
    NVML calls, the interpreter) then cannot leave the GPU idle between a step's start event and
    its launch, which would count as step time.  Every step's work stays inside its events; the
    callers run UNTIMED_AFTER_LEAD_IN untimed steps right after the lead-in (with one, the first
    timed step still ran 5-25 us slower than the median in nearly every run of the particle-filter
    step) and fill the flush buffer with non-zero values (a zero fill may take another path than
    the other steps')."""
    global _LEAD_IN_READY
    if not _LEAD_IN_READY:   # the spin kernel's first launch loads its module (host time): not here
        torch.cuda._sleep(1000)
        torch.cuda.synchronize()
        _LEAD_IN_READY = True
    torch.cuda._sleep(int(ms * 1e-3 * 2.0e9))


def _event_steps(torch, stream, steps, flush, step_fn):
    """CUDA-event time of each step (ms), L2 flushed before every step; returns (times, launches)."""
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    launches = 0
    torch.cuda.synchronize()
    gpu_lead_in(torch)
    for u in range(UNTIMED_AFTER_LEAD_IN):   # untimed: the first steps after the lead-in
        flush.fill_(-1.0 - u)
        step_fn()
    for k in range(steps):
        flush.fill_(float(k + 1))
        starts[k].record(stream)
        launches += step_fn()
        ends[k].record(stream)
    torch.cuda.synchronize()
    return [a.elapsed_time(b) for a, b in zip(starts, ends)], launches


def oracle_check_batch(rl, filters, host):
    """The batch's production weights (and ranges when kept) against the oracle on the host cores:
    bit for bit given the device's own per-ray cos/sin, and against the oracle with the host libm
    (the reference's own result here) the rays and particles that differ, all of them ones whose
    cos/sin differ."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    O.build(reference=False)
    nt = os.cpu_count() or 1
    t0 = time.perf_counter()
    res = {"filters": len(filters), "particles": 0, "bit_exact_given_same_trig": True, "trig_differs_rays": 0,
           "weights_differ_from_host_libm": 0, "weights_rel_diff_above_1e-6": 0, "explained_by_trig": True}
    for f, wl in zip(filters, host):
        meth, w = f[0], f[4].cpu().numpy()
        n, na = len(wl.ins), len(wl.angles)
        world = tuple(float(np.float32(v)) for v in wl.world)
        ref = O.OracleMethod(wl.occ, "rm", wl.max_range, world=world)
        ref.set_sensor_model(wl.table)
        xyh, trig_libm = O.world_rays(world, wl.ins, wl.angles)
        trig_cr = np.ascontiguousarray(rl.trig_eval(xyh[:, 2])[:, ::-1])
        del xyh
        tdiff = np.any(trig_cr.view(np.uint32) != trig_libm.view(np.uint32), axis=1)
        ref.set_trig_override(trig_cr)
        w_cr = ref.calc_range_repeat_angles_eval_sensor_model(wl.ins, wl.angles, wl.obs, nthreads=nt)
        ref.set_trig_override(None)
        w_libm = ref.calc_range_repeat_angles_eval_sensor_model(wl.ins, wl.angles, wl.obs, nthreads=nt)
        res["particles"] += n
        res["trig_differs_rays"] += int(tdiff.sum())
        res["bit_exact_given_same_trig"] &= bool(np.array_equal(w.view(np.uint64), w_cr.view(np.uint64)))
        wd = w.view(np.uint64) != w_libm.view(np.uint64)
        res["weights_differ_from_host_libm"] += int(wd.sum())
        res["explained_by_trig"] &= not bool(np.any(wd & ~tdiff.reshape(n, na).any(axis=1)))
        with np.errstate(divide="ignore", invalid="ignore"):
            rel = np.where(w_libm != 0, np.abs(w - w_libm) / np.abs(w_libm), np.where(w == 0, 0.0, np.inf))
        res["weights_rel_diff_above_1e-6"] += int(np.sum(rel > 1e-6))
    res["oracle_s"] = time.perf_counter() - t0
    res["oracle_threads"] = nt
    return res


def run_batch(args, emit=True, oracle_check=False):
    """32 uneven particle filters (maps 512-4096 px, 500-20,000 particles, 30-1,081 beams,
    max_range 100-400 px) updated by one persistent launch replayed as a CUDA graph, against
    per-filter plain calls (cast to ranges, then the sensor model, host buffers -- the
    reference's per-call pattern) and per-filter fused device calls.  Returns the JSON line
    (printed when `emit`); `oracle_check` adds the weights' check against the oracle."""
    import torch
    import range_libc_gb300.range_libc as rl
    from range_libc_gb300 import workloads as W

    rank, ws, dist = dist_init()
    dev = torch.device("cuda", torch.cuda.current_device())
    stream = torch.cuda.current_stream(dev)
    specs = W.uneven_batch_specs()[: args.filters]
    filters, host, keep = [], [], []
    t0 = time.perf_counter()
    for spec in specs:
        wl = W.batch_filter(spec)
        omap = rl.PyOMap(np.ascontiguousarray(wl.occ.T))
        m = rl.PyRayMarching(omap, wl.max_range)
        m.set_sensor_model(wl.table)
        t = [torch.from_numpy(a).to(dev) for a in (wl.ins, wl.angles, wl.obs)]
        w = torch.zeros(len(wl.ins), dtype=torch.float64, device=dev)
        filters.append((m, t[0], t[1], t[2], w))
        host.append(wl)
        keep.append(omap)
    torch.cuda.synchronize()
    setup_s = time.perf_counter() - t0
    rays = sum(len(wl.ins) * len(wl.angles) for wl in host)
    particles = sum(len(wl.ins) for wl in host)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    # per-filter schedules for the per-filter comparison, one batch schedule for the batch
    if not args.no_plain:
        for m, ins, ang, obs, w in filters:
            m.autotune(ins, ang, obs, w)
    batch = rl.PyFilterBatch(filters)
    if args.schedule:
        sched = [int(v) for v in args.schedule.split(",")]
        batch.set_schedule(*sched[:4])
        if len(sched) > 4:   # fifth field: products overlapped (0) or in a separate launch (1)
            batch.set_product_mode(bool(sched[4]))
    else:
        batch.autotune()

    def batched():
        batch.run()   # one graph: observation bins, the persistent cast (+ the products launch when separate)
        return 3 if batch.product_mode() == "separate" else 2

    def per_filter_fused():
        for m, ins, ang, obs, w in filters:
            m.calc_range_repeat_angles_eval_sensor_model(ins, ang, obs, w)
        return len(filters)

    for _ in range(args.warmup):
        batched()
    barrier(dist)
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    tb, launches = _event_steps(torch, stream, args.steps, flush, batched)
    clk = clocks.stop()
    ref_w = [f[4].cpu().numpy().copy() for f in filters]
    if args.no_plain:
        total_b = max_over_ranks(dist, sum(tb))
        short = {"metric": METRIC, "value": ws * rays * args.steps / (total_b / 1e3), "unit": "rays/s",
                 "ms_per_step": total_b / args.steps, "filters": len(filters), "rays_per_step": rays,
                 "gpu_launches": launches}
        if rank == 0 and emit:
            print(json.dumps(short))
        return short
    for _ in range(args.warmup):
        per_filter_fused()
    tf, _ = _event_steps(torch, stream, args.steps, flush, per_filter_fused)
    same = all(np.array_equal(f[4].cpu().numpy(), r) for f, r in zip(filters, ref_w))

    # plain per-filter calls through host buffers: cast to ranges, then the sensor model
    hbuf = [(wl.ins, wl.angles, wl.obs, np.empty(len(wl.ins) * len(wl.angles), np.float32),
             np.empty(len(wl.ins), np.float64)) for wl in host]

    def plain_host():
        for (m, *_), (hi, ha, ho, hr, hw) in zip(filters, hbuf):
            m.calc_range_repeat_angles(hi, ha, hr)
            m.eval_sensor_model(ho, hr, hw, len(ha), len(hi))

    plain_host()
    plain_steps = max(2, min(args.steps, 5))
    tp = 0.0
    for k in range(plain_steps):
        flush.fill_(float(k))
        torch.cuda.synchronize()
        a = time.perf_counter()
        plain_host()
        tp += time.perf_counter() - a
    same_plain = all(np.array_equal(h[4], r) for h, r in zip(hbuf, ref_w))

    total_b = max_over_ranks(dist, sum(tb))
    value = ws * rays * args.steps / (total_b / 1e3)
    # roofline of k_batch: per particle pose in + weight out, per ray one table read + a 2-byte
    # range bin written and read back + 4 B per distance-transform read
    steps_total = sum(m.count_steps(wl.ins, wl.angles) for (m, *_), wl in zip(filters, host))
    alg_bytes = particles * (12 + 8) + rays * (8 + 4) + 4 * steps_total
    peak, peak_kind = load_peaks()
    achieved = alg_bytes / (total_b / args.steps / 1e3) / 1e9
    traffic, traffic_src = BATCH_NCU_TRAFFIC.get(len(filters), (None, None))
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": traffic, "traffic_source": traffic_src,
                "peak_source": f"hbm_gbs burst ({peak_kind})", "algorithmic_bytes_per_launch": alg_bytes,
                "mean_march_steps_per_ray": steps_total / rays, "kernel": "k_batch (persistent cast + products)"}
    line = {
        "metric": METRIC, "value": value, "unit": "rays/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_b / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 ranges / f64 weights", "data": "synthetic",
        "config": {"workload": "32 uneven filters (maps 512-4096 px, RM), one persistent launch as a CUDA graph",
                   "filters": len(filters), "rays_per_step": rays, "particles_per_step": particles,
                   "schedule": dict(zip(("dt_layout", "prefetch", "block", "tile"), batch.schedule()),
                                    products=batch.product_mode()),
                   "l2": "flushed before every step (256 MiB write); maps total > L2"},
        "particle_updates_per_s": ws * particles * args.steps / (total_b / 1e3),
        "per_filter_fused_rays_per_s": rays * args.steps / (sum(tf) / 1e3),
        "plain_per_call_rays_per_s": rays * plain_steps / tp,
        "batched_over_plain": (rays * args.steps / (sum(tb) / 1e3)) / (rays * plain_steps / tp),
        "weights_equal_per_filter_fused": same, "weights_equal_plain": same_plain,
        "gpu_launches": launches, "setup_s": setup_s, "roofline": roofline, "clocks": clk,
    }
    if oracle_check and rank == 0:
        line["weights_vs_oracle"] = oracle_check_batch(rl, filters, host)
    if rank == 0 and emit:
        print(json.dumps(line))
        if args.out:
            with open(args.out, "w") as f:
                f.write(json.dumps(line) + "\n")
    return line


def run_cddt(args):
    """CDDT (or pruned CDDT) queries on a 2048^2 rectangles-and-disks map: GPU table build
    time and 1M-query throughput."""
    import torch
    import range_libc_gb300.range_libc as rl
    from range_libc_gb300 import workloads as W

    rank, ws, dist = dist_init()
    dev = torch.device("cuda", torch.cuda.current_device())
    stream = torch.cuda.current_stream(dev)
    wl = W.cddt_queries(td=args.td)
    omap = rl.PyOMap(np.ascontiguousarray(wl.occ.T))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    m = rl.PyCDDTCast(omap, wl.max_range, args.td)
    torch.cuda.synchronize()
    build_s = time.perf_counter() - t0
    prune_s = None
    if args.prune:
        t0 = time.perf_counter()
        m.prune()
        torch.cuda.synchronize()
        prune_s = time.perf_counter() - t0
    _, _, bin_len, zeros = m.table()
    ins = torch.from_numpy(wl.ins).to(dev)
    outs = torch.empty(len(wl.ins), dtype=torch.float32, device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def step():
        m.calc_range_many(ins, outs)
        return 1

    per_mode = {}
    for warp_search in (0, 1, 2):   # per-thread binary, warp-cooperative and sector bin search
        m.set_schedule(0, 0, warp_search, 0)
        for _ in range(args.warmup):
            step()
        t_mode, _ = _event_steps(torch, stream, args.steps, flush, step)
        per_mode[warp_search] = sum(t_mode)
    best = min(per_mode, key=per_mode.get)
    m.set_schedule(0, 0, best, 0)
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    t, launches = _event_steps(torch, stream, args.steps, flush, step)
    clk = clocks.stop()
    total = max_over_ranks(dist, sum(t))
    n = len(wl.ins)
    value = ws * n * args.steps / (total / 1e3)
    h_out = np.empty(n, np.float32)
    t0 = time.perf_counter()
    m.calc_range_many(wl.ins, h_out)
    e2e_s = time.perf_counter() - t0
    same = np.array_equal(h_out, outs.cpu().numpy())
    line = {
        "metric": METRIC, "value": value, "unit": "rays/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"{'PCDDT' if args.prune else 'CDDT'} td {args.td}, 2048^2 rect/disk map, "
                               f"{n} free-cell queries", "l2": "flushed before every step (256 MiB write)"},
        "table": {"build_s": build_s, "prune_s": prune_s, "bins": int(len(bin_len)), "zeros": int(len(zeros)),
                  "mean_bin": float(np.mean(bin_len)), "max_bin": int(np.max(bin_len))},
        "e2e": {"value": n / e2e_s, "unit": "rays/s", "h2d_bytes_per_step": wl.ins.nbytes,
                "d2h_bytes_per_step": h_out.nbytes},
        "host_equals_device": same, "gpu_launches": launches, "clocks": clk,
        "search": {"per_thread_rays_per_s": n * args.steps / (per_mode[0] / 1e3),
                   "warp_cooperative_rays_per_s": n * args.steps / (per_mode[1] / 1e3),
                   "sector_rays_per_s": n * args.steps / (per_mode[2] / 1e3), "chosen": int(best)},
    }
    if rank == 0:
        print(json.dumps(line))
        if args.out:
            with open(args.out, "w") as f:
                f.write(json.dumps(line) + "\n")
    return 0


def run_glt(args):
    """GiantLUTCast on the 2048^2 rectangles-and-disks map: GPU table build (one ray march per
    cell corner and angle bin) and 1M-query throughput."""
    import torch
    import range_libc_gb300.range_libc as rl
    from range_libc_gb300 import workloads as W

    rank, ws, dist = dist_init()
    dev = torch.device("cuda", torch.cuda.current_device())
    stream = torch.cuda.current_stream(dev)
    wl = W.cddt_queries(td=args.td)
    omap = rl.PyOMap(np.ascontiguousarray(wl.occ.T))
    rl.PyRayMarching(omap, wl.max_range)   # distance transform outside the build timing
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    m = rl.PyGiantLUTCast(omap, wl.max_range, args.td)
    torch.cuda.synchronize()
    build_s = time.perf_counter() - t0
    w, h = wl.occ.shape
    build_rays = w * h * args.td
    ins = torch.from_numpy(wl.ins).to(dev)
    outs = torch.empty(len(wl.ins), dtype=torch.float32, device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def step():
        m.calc_range_many(ins, outs)
        return 1

    for _ in range(args.warmup):
        step()
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    t, launches = _event_steps(torch, stream, args.steps, flush, step)
    clk = clocks.stop()
    total = max_over_ranks(dist, sum(t))
    n = len(wl.ins)
    value = ws * n * args.steps / (total / 1e3)
    peak, peak_kind = load_peaks()
    # per query: 12 B pose in, 4 B range out, one 2-byte table entry (a 32-B sector in practice)
    alg = n * (12 + 4 + 2)
    achieved = alg / (total / args.steps / 1e3) / 1e9
    line = {
        "metric": METRIC, "value": value, "unit": "rays/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u16 table / f32 ranges", "data": "synthetic",
        "config": {"workload": f"GiantLUTCast td {args.td}, 2048^2 rect/disk map, {n} free-cell queries",
                   "l2": "flushed before every step (256 MiB write); table > L2"},
        "table": {"build_s": build_s, "build_rays": build_rays, "build_rays_per_s": build_rays / build_s,
                  "bytes": build_rays * 2},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": None, "peak_source": f"hbm_gbs burst ({peak_kind})",
                     "algorithmic_bytes_per_launch": alg, "kernel": "k_calc_range_many<GLT>"},
        "gpu_launches": launches, "clocks": clk,
    }
    if rank == 0:
        print(json.dumps(line))
        if args.out:
            with open(args.out, "w") as f:
                f.write(json.dumps(line) + "\n")
    return 0


def run_radial(args):
    """CDDT calc_range_many_radial_optimized on the particle-filter step's map and poses (4,000
    particles x 61 beams over 270 degrees) against calc_range_repeat_angles of the same beams."""
    import torch
    import range_libc_gb300.range_libc as rl
    from range_libc_gb300 import workloads as W

    rank, ws, dist = dist_init()
    dev = torch.device("cuda", torch.cuda.current_device())
    stream = torch.cuda.current_stream(dev)
    wl = W.particle_filter_step()
    omap = rl.PyOMap(np.ascontiguousarray(wl.occ.T))
    omap.set_world(*wl.world[:4])
    m = rl.PyCDDTCast(omap, wl.max_range, args.td)
    if args.prune:
        m.prune()
    n, na = len(wl.ins), len(wl.angles)
    lo, hi = float(wl.angles[0]), float(wl.angles[-1])
    ins = torch.from_numpy(wl.ins).to(dev)
    ang = torch.from_numpy(wl.angles).to(dev)
    out_r = torch.empty(n * na, dtype=torch.float32, device=dev)
    out_a = torch.empty(n * na, dtype=torch.float32, device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def radial():
        m.calc_range_many_radial_optimized(na, lo, hi, ins, out_r)
        return 1

    def angles():
        m.calc_range_repeat_angles(ins, ang, out_a)
        return 1

    for _ in range(args.warmup):
        radial()
        angles()
    ta, _ = _event_steps(torch, stream, args.steps, flush, angles)
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    t, launches = _event_steps(torch, stream, args.steps, flush, radial)
    clk = clocks.stop()
    total = max_over_ranks(dist, sum(t))
    value = ws * n * na * args.steps / (total / 1e3)
    line = {
        "metric": METRIC, "value": value, "unit": "rays/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"{'PCDDT' if args.prune else 'CDDT'} td {args.td} radial pairs, corridor 2048^2 "
                               f"@0.05 m/px, {n} particles x {na} beams over 270 deg",
                   "l2": "flushed before every step (256 MiB write)"},
        "repeat_angles_rays_per_s": n * na * args.steps / (sum(ta) / 1e3),
        "radial_over_repeat_angles": sum(ta) / sum(t),
        "gpu_launches": launches, "clocks": clk,
    }
    if rank == 0:
        print(json.dumps(line))
        if args.out:
            with open(args.out, "w") as f:
                f.write(json.dumps(line) + "\n")
    return 0


def run_learned(args, emit=True):
    """Learned range surrogate on a 4096^2 rectangles-and-disks map: train on rays from the
    exact marcher, then 10,000 particles x 108 beams through the learned query (accept check +
    exact recast) against the exact path; range and weight errors on the same queries.  Returns
    the JSON line (printed when `emit`)."""
    import torch
    import range_libc_gb300.range_libc as rl
    from range_libc_gb300 import workloads as W

    rank, ws, dist = dist_init()
    dev = torch.device("cuda", torch.cuda.current_device())
    stream = torch.cuda.current_stream(dev)
    mr = 300.0
    occ = W.rect_disk_map(4096, 5000)
    omap = rl.PyOMap(np.ascontiguousarray(occ.T))
    rm = rl.PyRayMarching(omap, mr)
    K = int(mr) + 1
    table = W.sensor_table(K)
    rm.set_sensor_model(table)
    model = rl.PyLearnedRM(rm, seed=1)
    batch = args.train_batch
    steps = max(1, args.train_rays // batch)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    loss = model.train(steps=steps, batch=batch, lr=args.train_lr, seed=2)
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t0

    # held-out rays: hit-parameter error of the raw predictions
    xyt, t_true, _ = model.sample_rays(2_000_000, first_id=4_000_000_000 // 2, seed=77)
    pred = model.predict(xyt)
    e_t = (pred - t_true).abs().cpu().numpy()

    # the query workload: 10,000 particles x 108 beams, free-cell poses, uniform headings
    fs = W.free_cell_queries(occ, 10_000, 5001)
    ins_np = np.stack([fs[:, 1], fs[:, 0], fs[:, 2]], 1).astype(np.float32)   # world frame, identity map world
    ang_np = np.linspace(-np.pi, np.pi, 108, endpoint=False).astype(np.float32)
    obs_np = np.random.default_rng(5002).uniform(0, mr, 108).astype(np.float32)
    ins, ang, obs = (torch.from_numpy(a).to(dev) for a in (ins_np, ang_np, obs_np))
    n, na = len(ins_np), len(ang_np)
    out_l = torch.empty(n * na, dtype=torch.float32, device=dev)
    out_e = torch.empty(n * na, dtype=torch.float32, device=dev)
    acc = torch.empty(n * na, dtype=torch.uint8, device=dev)
    w_l = torch.empty(n, dtype=torch.float64, device=dev)
    w_e = torch.empty(n, dtype=torch.float64, device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    rm.autotune(ins, ang, obs, w_e)

    def exact_step():
        rm.calc_range_repeat_angles(ins, ang, out_e)
        return 1

    def exact_fused():
        rm.calc_range_repeat_angles_eval_sensor_model(ins, ang, obs, w_e)
        return 1

    n_recast = [0]

    def learned_step():
        n_recast[0] = model.calc_range_repeat_angles(ins, ang, out_l, acc)
        return 1

    for f in (exact_step, exact_fused, learned_step):
        for _ in range(args.warmup):
            f()
    te, _ = _event_steps(torch, stream, args.steps, flush, exact_step)
    tf, _ = _event_steps(torch, stream, args.steps, flush, exact_fused)
    tl, _ = _event_steps(torch, stream, args.steps, flush, learned_step)
    rm.eval_sensor_model(obs, out_l, w_l, na, n)
    torch.cuda.synchronize()
    ol, oe = out_l.cpu().numpy(), out_e.cpu().numpy()
    a = acc.cpu().numpy().astype(bool)
    err = np.abs(ol - oe)
    wl_, we_ = w_l.cpu().numpy(), w_e.cpu().numpy()
    pos = (we_ > 0) & (wl_ > 0)
    rel_w = np.abs(wl_[pos] - we_[pos]) / we_[pos]
    logw = np.abs(np.log(wl_[pos]) - np.log(we_[pos]))
    rays = n * na
    line = {
        "metric": METRIC, "value": rays * args.steps / (sum(tl) / 1e3), "unit": "rays/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": sum(tl) / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "bf16 MLP (fp32 accumulate) + f32 exact recast",
        "data": "synthetic",
        "config": {"workload": "learned surrogate, 4096^2 rect/disk map, RM max_range 300 px, 10,000 particles x 108 "
                               "beams; MLP 512 Fourier features -> 4 x 256 GELU -> 1",
                   "train_rays": steps * batch, "train_batch": batch, "train_s": train_s, "final_loss": loss,
                   "train_rays_per_s": steps * batch / train_s},
        "exact_repeat_angles_rays_per_s": rays * args.steps / (sum(te) / 1e3),
        "exact_fused_rays_per_s": rays * args.steps / (sum(tf) / 1e3),
        "learned_over_exact": (sum(te) / sum(tl)),
        "fallback_rate": n_recast[0] / rays,
        "heldout_t_error_px": {"median": float(np.median(e_t)), "p99": float(np.percentile(e_t, 99))},
        "range_error_px_all": {"median": float(np.median(err)), "p99": float(np.percentile(err, 99))},
        "range_error_px_accepted": {"median": float(np.median(err[a])) if a.any() else None,
                                    "p99": float(np.percentile(err[a], 99)) if a.any() else None,
                                    "exact_fraction": float(np.mean(err[a] == 0)) if a.any() else None},
        "weight_error": {"median_rel": float(np.median(rel_w)) if len(rel_w) else None,
                         "p99_rel": float(np.percentile(rel_w, 99)) if len(rel_w) else None,
                         "median_abs_log": float(np.median(logw)) if len(logw) else None},
        "gpu_launches": None,
    }
    if rank == 0 and emit:
        print(json.dumps(line))
        if args.out:
            with open(args.out, "w") as f:
                f.write(json.dumps(line) + "\n")
    return line


if __name__ == "__main__":
    sys.exit(main())
