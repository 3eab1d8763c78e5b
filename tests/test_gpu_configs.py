"""The four benchmarked workloads at their full sizes, on the GPU, against the oracle.

Each workload is built with the same generators and seeds as bench.py:

  1. BL and RM calc_range_many: 512^2 rectangles-and-disks map, 10,000 free-cell queries,
     max_range 300 (RangeLib.h:439-480, 696-769, 927-962);
  2. one particle-filter step: 2048^2 corridor at 0.05 m/px, 4,000 particles x 61 beams,
     max_range 200, 201 x 201 sensor table -- the fused call and the cast followed by
     eval_sensor_model (RangeLib.h:482-612), under the autotuned schedule and two fixed ones;
  3. CDDT and pruned CDDT at theta_discretization 108 and 216 on a 2048^2 map: the GPU-built
     tables and 1,000,000 queries under each bin search (RangeLib.h:974-1516);
  4. 32 uneven ray-marching filters (maps 512-4096 px, 500-20,000 particles, 30-1,081 beams)
     through one persistent launch, ranges and weights.

Two modes are checked for the casts that take a per-ray cos/sin (BL, RM):

  * parity: the oracle's own per-ray cosf/sinf (the host libm's, as the reference) fed to the
    GPU -- ranges and weights must be bit-identical to the oracle's;
  * production (no override): the GPU uses the correctly rounded cos/sin (rlc_trig_eval).
    Its ranges and weights must be bit-identical to the oracle fed those same values, and
    against the oracle with the host libm (the reference's own result on this host) every
    differing ray or particle must be one whose cos/sin differ between the two.  The counts are
    printed ("PARITY ..." lines, pytest -s): the target tolerances (hit cells exact, RM
    within 1e-4 px, weights within 1e-6 relative) hold on every other ray and particle.

CDDT needs only the cos/sin of its slice angles, which both sides take from the host libm, so
its queries are compared bit for bit in one mode.
"""
import os

import numpy as np
import pytest

from range_libc_gb300 import workloads as W

pytestmark = pytest.mark.gpu
NT = os.cpu_count() or 1


def _bits(a):
    a = np.ascontiguousarray(a)
    return a.view(np.uint32 if a.dtype == np.float32 else np.uint64)


def _trig_cr(rl, headings):
    """(cos, sin) the production casts use for each heading, computed by the device."""
    h = np.ascontiguousarray(headings, np.float32)
    sc = np.empty((len(h), 2), np.float32)
    rl._lib.call("rlc_trig_eval", h.ctypes.data, sc.ctypes.data, len(h), 0, None)
    return np.ascontiguousarray(sc[:, ::-1])


def _rays(oracle_mod, rl, world, ins, angles=None):
    """Per ray: the host libm's (cos, sin), the production (cos, sin), and whether they differ."""
    xyh, trig_libm = oracle_mod.world_rays(world, ins, angles)
    trig_cr = _trig_cr(rl, xyh[:, 2])
    diff = np.any(_bits(trig_cr) != _bits(trig_libm), axis=1)
    return trig_libm, trig_cr, diff


def _report(tag, **kw):
    print("PARITY " + tag + " " + " ".join(f"{k}={v}" for k, v in kw.items()), flush=True)


def _check_ranges(tag, got, exp_cr, exp_libm, trig_diff, tol_px=None, scale=1.0):
    """Production ranges: exact against the oracle fed the same cos/sin; against the oracle with
    the host libm, differences only on rays whose cos/sin differ."""
    assert np.array_equal(_bits(got), _bits(exp_cr)), \
        f"{tag}: {int(np.sum(_bits(got) != _bits(exp_cr)))} ranges differ from the oracle given the same cos/sin"
    diff = _bits(got) != _bits(exp_libm)
    assert not np.any(diff & ~trig_diff), f"{tag}: a range differs on a ray whose cos/sin agree"
    dev = np.abs(got.astype(np.float64) - exp_libm.astype(np.float64)) / scale
    out_tol = int(np.sum(dev > tol_px)) if tol_px is not None else int(np.sum(diff))
    _report(tag, rays=len(got), trig_differs=int(trig_diff.sum()), ranges_differ=int(diff.sum()),
            out_of_tolerance=out_tol, max_abs_px=float(dev.max()) if len(dev) else 0.0)
    return out_tol


def _check_weights(tag, got, exp_cr, exp_libm, particle_trig_diff):
    assert np.array_equal(_bits(got), _bits(exp_cr)), \
        f"{tag}: {int(np.sum(_bits(got) != _bits(exp_cr)))} weights differ from the oracle given the same cos/sin"
    diff = _bits(got) != _bits(exp_libm)
    assert not np.any(diff & ~particle_trig_diff), f"{tag}: a weight differs on a particle whose cos/sin all agree"
    with np.errstate(divide="ignore", invalid="ignore"):
        rel = np.where(exp_libm != 0, np.abs(got - exp_libm) / np.abs(exp_libm), np.where(got == 0, 0.0, np.inf))
    out_tol = int(np.sum(rel > 1e-6))
    _report(tag, particles=len(got), with_trig_diff=int(particle_trig_diff.sum()), weights_differ=int(diff.sum()),
            rel_diff_above_1e6=out_tol)
    return out_tol


# ------------------------------------------------------------------ workload 1
@pytest.mark.parametrize("kind", ["bl", "rm"])
def test_rect_disk_512_calc_range_many(rl, oracle_mod, kind):
    wl = W.rect_disk_queries(side=512, n=10_000, max_range=300.0, seed=1000)
    m = rl.PyOMap(np.ascontiguousarray(wl.occ.T))
    meth = (rl.PyBresenhamsLine if kind == "bl" else rl.PyRayMarching)(m, wl.max_range)
    ref = oracle_mod.OracleMethod(wl.occ, kind, wl.max_range, world=m.world)
    trig_libm, trig_cr, tdiff = _rays(oracle_mod, rl, m.world, wl.ins)
    exp_libm = ref.calc_range_many(wl.ins, nthreads=NT)
    out = np.empty(len(wl.ins), np.float32)
    meth.set_trig_override(trig_libm)                         # parity mode
    meth.calc_range_many(wl.ins, out)
    assert np.array_equal(_bits(out), _bits(exp_libm))
    meth.set_trig_override(None)                              # production
    meth.calc_range_many(wl.ins, out)
    ref.set_trig_override(trig_cr)
    exp_cr = ref.calc_range_many(wl.ins, nthreads=NT)
    _check_ranges(f"config1 {kind} calc_range_many", out, exp_cr, exp_libm, tdiff,
                  tol_px=1e-4 if kind == "rm" else None)


# ------------------------------------------------------------------ workload 2
@pytest.fixture(scope="module")
def pf_full():
    return W.particle_filter_step()   # bench.py's particle-filter step (seed 2000)


def test_particle_filter_step_2048_4000x61(rl, oracle_mod, pf_full):
    torch = pytest.importorskip("torch")
    wl = pf_full
    n, na = len(wl.ins), len(wl.angles)
    m = rl.PyOMap(np.ascontiguousarray(wl.occ.T))
    m.set_world(*wl.world[:4])
    meth = rl.PyRayMarchingGPU(m, wl.max_range)
    meth.set_sensor_model(wl.table)
    ref = oracle_mod.OracleMethod(wl.occ, "rm", wl.max_range, world=m.world)
    ref.set_sensor_model(wl.table)
    trig_libm, trig_cr, tdiff = _rays(oracle_mod, rl, m.world, wl.ins, wl.angles)
    pdiff = tdiff.reshape(n, na).any(axis=1)
    exp = {}
    for mode, trig in (("libm", None), ("cr", trig_cr)):
        ref.set_trig_override(trig)
        exp[mode] = (ref.calc_range_repeat_angles_eval_sensor_model(wl.ins, wl.angles, wl.obs, nthreads=NT),
                     ref.calc_range_repeat_angles(wl.ins, wl.angles, nthreads=NT))
    ref.set_trig_override(None)
    # eval_sensor_model bins world ranges (px * scale * inv_scale), so it may differ from the fused
    # call's pixel bins; each is compared with the oracle's own
    exp_eval = {k: ref.eval_sensor_model(wl.obs, v[1], na, n, nthreads=NT) for k, v in exp.items()}

    dev = torch.device("cuda:0")
    t = [torch.from_numpy(a).to(dev) for a in (wl.ins, wl.angles, wl.obs)]
    tw = torch.empty(n, dtype=torch.float64, device=dev)
    meth.autotune(t[0], t[1], t[2], tw, flush_l2=True)
    tuned = meth.schedule()
    table = meth.autotune_results()
    finalists = [sched for sched, _, final in table if final is not None]
    assert len(finalists) == 3 and any(f[0] == tuned[0] and f[2:] == tuned[2:] for f in finalists)
    w = np.empty(n, np.float64)
    r = np.empty(n * na, np.float32)
    we = np.empty(n, np.float64)
    for sched in (tuned, (0, 0, 0, 0), (4, 0, 0, 0), (5, 0, 0, 0), (2, 0, 1, 0)):
        meth.set_schedule(*sched)
        meth.set_trig_override(trig_libm)                     # parity mode
        meth.calc_range_repeat_angles_eval_sensor_model(wl.ins, wl.angles, wl.obs, w)
        assert np.array_equal(_bits(w), _bits(exp["libm"][0])), sched
        meth.calc_range_repeat_angles(wl.ins, wl.angles, r)
        assert np.array_equal(_bits(r), _bits(exp["libm"][1])), sched
        meth.eval_sensor_model(wl.obs, r, we, na, n)
        assert np.array_equal(_bits(we), _bits(exp_eval["libm"])), sched
        meth.set_trig_override(None)                          # production
        meth.calc_range_repeat_angles_eval_sensor_model(wl.ins, wl.angles, wl.obs, w)
        _check_weights(f"config2 fused schedule={tuple(sched)}", w, exp["cr"][0], exp["libm"][0], pdiff)
        meth.calc_range_repeat_angles(wl.ins, wl.angles, r)
        _check_ranges(f"config2 calc_range_repeat_angles schedule={tuple(sched)}", r, exp["cr"][1],
                      exp["libm"][1], tdiff, tol_px=1e-4, scale=wl.world[0])
        meth.eval_sensor_model(wl.obs, r, we, na, n)
        _check_weights(f"config2 cast + eval_sensor_model schedule={tuple(sched)}", we, exp_eval["cr"],
                       exp_eval["libm"], pdiff)


# ------------------------------------------------------------------ workload 3
@pytest.mark.parametrize("td", [108, 216])
def test_cddt_and_pcddt_2048_1m_queries(rl, oracle_mod, td):
    wl = W.cddt_queries(side=2048, n=1_000_000, td=td)
    m = rl.PyOMap(np.ascontiguousarray(wl.occ.T))
    for pruned in (False, True):
        g = rl.PyCDDTCast(m, wl.max_range, td)
        ref = oracle_mod.OracleMethod(wl.occ, "pcddt" if pruned else "cddt", wl.max_range, td=td)
        if pruned:
            g.prune()
        gw, gt, gl, gz = g.table()
        rw, rt, rlen, rz = ref.cddt_table()
        assert np.array_equal(gw, rw) and np.array_equal(_bits(gt), _bits(rt))
        assert np.array_equal(gl, rlen) and np.array_equal(_bits(gz), _bits(rz))
        exp = ref.calc_range_many(wl.ins, nthreads=NT)
        out = np.empty(len(wl.ins), np.float32)
        for search in (0, 1, 2):   # binary, warp-cooperative and sector bin search
            g.set_schedule(0, 0, search, 0)
            out.fill(-1.0)
            g.calc_range_many(wl.ins, out)
            assert np.array_equal(_bits(out), _bits(exp)), (pruned, search)
        _report(f"config3 {'pcddt' if pruned else 'cddt'} td={td}", queries=len(exp), zero_points=len(gz),
                ranges_differ=0)


# ------------------------------------------------------------------ workload 4
def test_uneven_batch_32_filters(rl, oracle_mod):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda:0")
    specs = W.uneven_batch_specs()
    filters, host, keep, exp, tr = [], [], [], [], []
    for spec in specs:
        wl = W.batch_filter(spec)
        omap = rl.PyOMap(np.ascontiguousarray(wl.occ.T))
        meth = rl.PyRayMarching(omap, wl.max_range)
        meth.set_sensor_model(wl.table)
        n, na = len(wl.ins), len(wl.angles)
        t = [torch.from_numpy(a).to(dev) for a in (wl.ins, wl.angles, wl.obs)]
        tw = torch.zeros(n, dtype=torch.float64, device=dev)
        tr_ = torch.zeros(n * na, dtype=torch.float32, device=dev)
        filters.append((meth, t[0], t[1], t[2], tw, tr_))
        keep.append(omap)
        host.append(wl)
        ref = oracle_mod.OracleMethod(wl.occ, "rm", wl.max_range, world=omap.world)
        ref.set_sensor_model(wl.table)
        trig_libm, trig_cr, tdiff = _rays(oracle_mod, rl, omap.world, wl.ins, wl.angles)
        e = {}
        for mode, trig in (("libm", None), ("cr", trig_cr)):
            ref.set_trig_override(trig)
            rng = ref.calc_range_repeat_angles(wl.ins, wl.angles, nthreads=NT)
            e[mode] = (rng, ref.eval_sensor_model(wl.obs, rng, na, n, nthreads=NT))
        exp.append(e)
        tr.append((trig_libm, tdiff))
        del ref, trig_cr
    rays = sum(len(w.ins) * len(w.angles) for w in host)
    batch = rl.PyFilterBatch(filters)
    batch.autotune()
    for mode in ("production", "parity"):
        for f, (trig_libm, _) in zip(filters, tr):
            f[0].set_trig_override(trig_libm if mode == "parity" else None)
        for f in filters:
            f[4].zero_()
            f[5].fill_(-1.0)
        batch.run()
        torch.cuda.synchronize()
        n_trig = n_rdiff = n_wdiff = n_wtol = 0
        for f, wl, e, (_, tdiff) in zip(filters, host, exp, tr):
            n, na = len(wl.ins), len(wl.angles)
            r = f[5].cpu().numpy()
            w = f[4].cpu().numpy()
            if mode == "parity":
                assert np.array_equal(_bits(r), _bits(e["libm"][0])) and np.array_equal(_bits(w), _bits(e["libm"][1]))
                continue
            assert np.array_equal(_bits(r), _bits(e["cr"][0])) and np.array_equal(_bits(w), _bits(e["cr"][1]))
            rd = _bits(r) != _bits(e["libm"][0])
            assert not np.any(rd & ~tdiff)
            pd = tdiff.reshape(n, na).any(axis=1)
            wd = _bits(w) != _bits(e["libm"][1])
            assert not np.any(wd & ~pd)
            with np.errstate(divide="ignore", invalid="ignore"):
                ref_w = e["libm"][1]
                rel = np.where(ref_w != 0, np.abs(w - ref_w) / np.abs(ref_w), np.where(w == 0, 0.0, np.inf))
            n_trig += int(tdiff.sum())
            n_rdiff += int(rd.sum())
            n_wdiff += int(wd.sum())
            n_wtol += int(np.sum(rel > 1e-6))
        if mode == "production":
            _report("config4 batch", filters=len(filters), rays=rays, trig_differs=n_trig, ranges_differ=n_rdiff,
                    weights_differ=n_wdiff, weights_rel_diff_above_1e6=n_wtol,
                    schedule=",".join(map(str, batch.schedule())), products=batch.product_mode())
    for f in filters:
        f[0].set_trig_override(None)
