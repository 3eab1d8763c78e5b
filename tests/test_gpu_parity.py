"""Parity of the CUDA library against the CPU oracle on the same inputs.

Bit-exact for the distance transform, the edge map, the CDDT tables and
every range and weight when the per-ray cos/sin of BL and RM are the
oracle's (parity mode).  With the device's own sincosf, ranges may differ
where a last-bit difference of cos/sin moves a ray across a cell corner;
that is bounded below.
"""
import os

import numpy as np
import pytest

from range_libc_gb300 import workloads as W

pytestmark = pytest.mark.gpu

MAPS = {}


def _map(name):
    if name in MAPS:
        return MAPS[name]
    if name == "single_occ":
        occ = np.ones((1, 1), np.uint8)
    elif name == "single_free":
        occ = np.zeros((1, 1), np.uint8)
    elif name == "quad":
        occ = np.array([[1, 0], [0, 0]], np.uint8)
    elif name == "small_5x6":
        occ = (np.random.default_rng(3).random((5, 6)) < 0.3).astype(np.uint8)
    elif name == "empty_40x25":
        occ = np.zeros((40, 25), np.uint8)
    elif name == "rect_128":
        occ = W.rect_disk_map(128, 21)
    elif name == "rect_200x120":
        occ = np.ascontiguousarray(W.rect_disk_map(256, 22)[:200, :120])
    elif name == "corridor_512":
        occ = W.corridor_map(512, 23)
    else:
        raise KeyError(name)
    MAPS[name] = occ
    return occ


def _pymap(rl, occ, world=None):
    m = rl.PyOMap(np.ascontiguousarray(occ.T))
    assert np.array_equal(m.occupancy, occ)
    if world is not None:
        m.set_world(*world[:4])
    return m


def _queries(occ, n, seed, spread=0.0):
    rng = np.random.default_rng(seed)
    W_, H_ = occ.shape
    q = np.empty((n, 3), np.float32)
    q[:, 0] = rng.uniform(-spread, W_ + spread, n)
    q[:, 1] = rng.uniform(-spread, H_ + spread, n)
    q[:, 2] = rng.uniform(-7.0, 7.0, n)
    return q


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint32 if a.dtype == np.float32 else np.uint64)


ALL_MAPS = ["single_occ", "single_free", "quad", "small_5x6", "empty_40x25", "rect_128", "rect_200x120",
            "corridor_512"]


@pytest.mark.parametrize("name", ALL_MAPS)
def test_distance_transform_and_edge_map(rl, oracle_mod, name):
    occ = _map(name)
    m = _pymap(rl, occ)
    dt = np.empty(occ.shape, np.float32)
    rl._lib.call("rlc_map_distance_transform", m.handle, dt.ctypes.data_as(rl._lib._f32p))
    assert np.array_equal(_bits(dt), _bits(oracle_mod.edt(occ)))
    edge = np.empty(occ.shape, np.uint8)
    rl._lib.call("rlc_map_edge_map", m.handle, edge.ctypes.data_as(rl._lib._u8p))
    assert np.array_equal(edge, oracle_mod.edge_map(occ))


def test_distance_transform_large_map(rl, oracle_mod):
    # 2048^2: the pass-2 sums f + q^2 exceed 2^24 and round in float
    occ = W.rect_disk_map(2048, 31)
    m = _pymap(rl, occ)
    dt = np.empty(occ.shape, np.float32)
    rl._lib.call("rlc_map_distance_transform", m.handle, dt.ctypes.data_as(rl._lib._f32p))
    assert np.array_equal(_bits(dt), _bits(oracle_mod.edt(occ)))


def _edt_cases():
    rng = np.random.default_rng(91)
    cases = []
    # both sides <= 4096: closed-form columns and shared-memory rows; a side in (4096, 16384]:
    # integer comparisons with the stacks in global memory; a side above 16384: the double F-H
    for w, h in ((4096, 40), (40, 4096), (4097, 40), (40, 4100), (16384, 9), (16385, 8), (8, 16390)):
        occ = (rng.random((w, h)) < 0.002).astype(np.uint8)
        cases.append((f"{w}x{h}", occ))
    occ = np.zeros((10976, 64), np.uint8)   # keys up to ~2^27 that round in float
    occ[0, 0] = 1
    occ[rng.integers(0, 10976, 5), rng.integers(0, 64, 5)] = 1
    cases.append(("10976x64_sparse", occ))
    # the limit: one corner obstacle, squared distances up to 2 * 4095^2 and keys near 2^25
    occ = np.zeros((4096, 4096), np.uint8)
    occ[0, 0] = 1
    occ[rng.integers(0, 4096, 20), rng.integers(0, 4096, 20)] = 1
    cases.append(("4096x4096_sparse", occ))
    # mostly empty columns: pass 2 meets FLT_MAX inputs and compares them in double
    occ = np.zeros((1500, 1300), np.uint8)
    for x in rng.integers(0, 1500, 3):
        occ[x, rng.integers(0, 1300, 4)] = 1
    cases.append(("empty_columns", occ))
    return cases


@pytest.mark.parametrize("name,occ", _edt_cases(), ids=[c[0] for c in _edt_cases()])
def test_distance_transform_both_paths(rl, oracle_mod, name, occ):
    m = _pymap(rl, occ)
    dt = np.empty(occ.shape, np.float32)
    rl._lib.call("rlc_map_distance_transform", m.handle, dt.ctypes.data_as(rl._lib._f32p))
    assert np.array_equal(_bits(dt), _bits(oracle_mod.edt(occ))), name


WORLDS = {
    "identity": (1.0, 0.0, 0.0, 0.0),
    "ros": (0.05, 0.0, -3.25, -1.5),
    "rotated": (0.1, 0.7, 2.0, -1.0),
}


@pytest.mark.parametrize("kind", ["bl", "rm"])
@pytest.mark.parametrize("name", ["small_5x6", "rect_128", "rect_200x120", "corridor_512"])
@pytest.mark.parametrize("wname", list(WORLDS))
def test_calc_range_many_parity_mode(rl, oracle_mod, kind, name, wname):
    occ = _map(name)
    m = _pymap(rl, occ, WORLDS[wname])
    mr = 120.0
    cls = rl.PyBresenhamsLine if kind == "bl" else rl.PyRayMarching
    g = cls(m, mr)
    ref = oracle_mod.OracleMethod(occ, kind, mr, world=m.world)
    s = m.world[0]
    q = _queries(occ, 4000, 5, spread=3.0)
    q[:, :2] *= s
    _, trig = oracle_mod.world_rays(m.world, q)
    g.set_trig_override(trig)
    out = np.empty(len(q), np.float32)
    g.calc_range_many(q, out)
    assert np.array_equal(_bits(out), _bits(ref.calc_range_many(q)))
    # raw calc_range semantics (no world transform)
    qr = _queries(occ, 4000, 6, spread=3.0)
    trig_raw = np.stack([np.cos(qr[:, 2].astype(np.float64)), np.sin(qr[:, 2].astype(np.float64))], 1)
    trig_raw = trig_raw.astype(np.float32)
    g.set_trig_override(trig_raw)
    out2 = np.empty(len(qr), np.float32)
    rl._lib.call("rlc_calc_range_many", g.handle, qr.ctypes.data, out2.ctypes.data, len(qr), rl._lib.RLC_NO_WORLD,
                 None)
    exp2 = np.array([ref.calc_range_trig(float(a), float(b), float(c), float(d))
                     for (a, b, _), (c, d) in zip(qr, trig_raw)], np.float32)
    assert np.array_equal(_bits(out2), _bits(exp2))


@pytest.mark.parametrize("kind", ["bl", "rm"])
def test_calc_range_many_device_trig(rl, oracle_mod, kind):
    """Device sincosf: ranges equal the oracle's except where cos/sin differ in the last bit."""
    occ = _map("corridor_512")
    m = _pymap(rl, occ)
    g = (rl.PyBresenhamsLine if kind == "bl" else rl.PyRayMarching)(m, 300.0)
    ref = oracle_mod.OracleMethod(occ, kind, 300.0)
    q = W.free_cell_queries(occ, 100_000, 9)
    out = np.empty(len(q), np.float32)
    g.calc_range_many(q, out)
    exp = ref.calc_range_many(q)
    frac = np.mean(_bits(out) != _bits(exp))
    assert frac < 1e-3, f"{frac:.2e} of rays differ"


@pytest.mark.parametrize("kind", ["bl", "rm", "cddt"])
def test_repeat_angles_parity(rl, oracle_mod, kind):
    occ = _map("corridor_512")
    world = WORLDS["ros"]
    m = _pymap(rl, occ, world)
    mr = 150.0
    if kind == "cddt":
        g = rl.PyCDDTCast(m, mr, 108)
    else:
        g = (rl.PyBresenhamsLine if kind == "bl" else rl.PyRayMarching)(m, mr)
    ref = oracle_mod.OracleMethod(occ, kind, mr, td=108, world=m.world)
    fs = W.free_cell_queries(occ, 300, 12)
    xw, yw = W.grid_to_world(fs[:, 0], fs[:, 1], m.world)
    ins = np.stack([xw, yw, fs[:, 2]], 1).astype(np.float32)
    angles = W.laser_angles(61)
    if kind != "cddt":
        _, trig = oracle_mod.world_rays(m.world, ins, angles)
        g.set_trig_override(trig)
    out = np.empty(len(ins) * len(angles), np.float32)
    g.calc_range_repeat_angles(ins, angles, out)
    exp = ref.calc_range_repeat_angles(ins, angles)
    assert np.array_equal(_bits(out), _bits(exp))
    if kind == "cddt":   # warp-cooperative bin search
        g.set_schedule(0, 0, 1, 0)
        g.calc_range_repeat_angles(ins, angles, out)
        assert np.array_equal(_bits(out), _bits(exp))
    if kind == "rm":     # every distance-transform layout, with and without prefetch
        for layout in (0, 1, 2, 4, 5):
            for pf in (0, 1):
                g.set_schedule(layout, 0, pf, 0)
                g.calc_range_repeat_angles(ins, angles, out)
                assert np.array_equal(_bits(out), _bits(exp)), (layout, pf)


def _corridors(W_, H_, seed):
    """Walls along x every 3-9 rows with door gaps: most march steps read distances 1, 2 and 3."""
    rng = np.random.default_rng(seed)
    occ = np.zeros((W_, H_), np.uint8)
    occ[:, :2] = occ[:, -2:] = 1
    y = 2
    while y < H_ - 4:
        y += int(rng.integers(3, 10))
        occ[2:W_ - 2, y:y + 1] = 1
        for _ in range(3):
            g0 = int(rng.integers(2, W_ - 12))
            occ[g0:g0 + int(rng.integers(3, 9)), y] = 0
    return occ


@pytest.mark.parametrize("mr", [6.0, 8.5, 9.998, 10.0, 31.7, 150.0, 1000.0])
def test_narrow_corridor_parity(rl, oracle_mod, mr):
    """Rays along corridors 2-8 px wide -- long chains of 1 px steps, the longest rays of a
    particle-filter step -- that end on walls, leave the map or reach max_range after a fractional
    step; every layout and prefetch, per-ray and fused calls, against the oracle."""
    occ = _corridors(420, 300, 7)
    m = _pymap(rl, occ)
    g = rl.PyRayMarching(m, mr)
    ref = oracle_mod.OracleMethod(occ, "rm", mr, world=m.world)
    rng = np.random.default_rng(8)
    fs = W.free_cell_queries(occ, 6000, 13)
    head = np.where(rng.random(len(fs)) < 0.7,
                    rng.integers(0, 4, len(fs)) * (np.pi / 2) + rng.normal(0, 0.02, len(fs)),
                    rng.uniform(-np.pi, np.pi, len(fs)))
    q = np.stack([fs[:, 0], fs[:, 1], head], 1).astype(np.float32)
    q[:200, 0] = rng.uniform(-3, 3, 200)            # near and beyond the map's edge
    q[200:400, 1] = rng.uniform(296, 303, 200)
    _, trig = oracle_mod.world_rays(m.world, q)
    exp = ref.calc_range_many(q)
    table = W.sensor_table(int(mr) + 1 if mr < 400 else 201)
    g.set_sensor_model(table)
    ref.set_sensor_model(table)
    angles = W.laser_angles(31)
    ins = q[:500]
    _, trig_a = oracle_mod.world_rays(m.world, ins, angles)
    obs = (np.linspace(1, 30, 31) % mr).astype(np.float32)
    exp_w = ref.calc_range_repeat_angles_eval_sensor_model(ins, angles, obs)
    for layout in (0, 1, 2, 4, 5):
        for pf in (0, 1):
            g.set_schedule(layout, 0, pf, 0)
            g.set_trig_override(trig)
            out = np.empty(len(q), np.float32)
            g.calc_range_many(q, out)
            assert np.array_equal(_bits(out), _bits(exp)), (layout, pf)
            g.set_trig_override(trig_a)
            w = np.empty(len(ins), np.float64)
            g.calc_range_repeat_angles_eval_sensor_model(ins, angles, obs, w)
            assert np.array_equal(_bits(w), _bits(exp_w)), (layout, pf)


@pytest.mark.parametrize("name", ["quad", "small_5x6", "rect_128", "rect_200x120", "corridor_512"])
@pytest.mark.parametrize("td", [16, 108, 107, 216])
def test_cddt_table_and_queries(rl, oracle_mod, name, td):
    occ = _map(name)
    m = _pymap(rl, occ)
    mr = 100.0
    for pruned in (False, True):
        g = rl.PyCDDTCast(m, mr, td)
        ref = oracle_mod.OracleMethod(occ, "cddt", mr, td=td)
        if pruned:
            g.prune()
            ref.prune()
        gw, gt, gl, gz = g.table()
        rw, rt, rlen, rz = ref.cddt_table()
        assert np.array_equal(gw, rw) and np.array_equal(_bits(gt), _bits(rt))
        assert np.array_equal(gl, rlen)
        assert np.array_equal(_bits(gz), _bits(rz))
        q = W.free_cell_queries(occ, 3000, 4) if occ.min() == 0 else _queries(occ, 3000, 4)
        q[:, 2] = np.random.default_rng(td).uniform(-10, 10, len(q))
        exp = ref.calc_range_many(q)
        for warp_search in (0, 1, 2):   # binary, warp-cooperative and sector bin search
            g.set_schedule(0, 0, warp_search, 0)
            out = np.empty(len(q), np.float32)
            g.calc_range_many(q, out)
            assert np.array_equal(_bits(out), _bits(exp)), warp_search


@pytest.mark.parametrize("side,td,prune", [(1024, 108, False), (1024, 107, True), (2048, 216, False)])
def test_cddt_sector_search_long_bins(rl, oracle_mod, side, td, prune):
    """The sector bin search where bins hold hundreds of zero points (rectangles-and-disks maps,
    up to ~2000 per bin): every search schedule against the oracle (1024^2) or against the binary
    search on 1M queries (2048^2), per-ray and repeat-angle calls."""
    wl = W.cddt_queries(side=side, n=200_000 if side == 1024 else 1_000_000, td=td)
    m = _pymap(rl, wl.occ)
    g = rl.PyCDDTCast(m, 300.0, td)
    if prune:
        g.prune()
    assert np.max(g.table()[2]) > 64   # bins long enough for several sector steps
    if side == 1024:
        ref = oracle_mod.OracleMethod(wl.occ, "pcddt" if prune else "cddt", 300.0, td=td, nthreads=os.cpu_count() or 1)
        exp = ref.calc_range_many(wl.ins[:50_000], nthreads=os.cpu_count() or 1)
    outs = {}
    for mode in (0, 1, 2):
        g.set_schedule(0, 0, mode, 0)
        out = np.empty(len(wl.ins), np.float32)
        g.calc_range_many(wl.ins, out)
        outs[mode] = out
        if side == 1024:
            assert np.array_equal(_bits(out[:50_000]), _bits(exp)), mode
    assert np.array_equal(_bits(outs[2]), _bits(outs[0])) and np.array_equal(_bits(outs[1]), _bits(outs[0]))
    angles = W.laser_angles(31)
    ra = {}
    for mode in (0, 2):
        g.set_schedule(0, 0, mode, 0)
        r = np.empty(2000 * 31, np.float32)
        g.calc_range_repeat_angles(wl.ins[:2000], angles, r)
        ra[mode] = r
    assert np.array_equal(_bits(ra[0]), _bits(ra[2]))


def test_cddt_given_table(rl, oracle_mod):
    """Queries over a table loaded from outside equal the oracle's over the same table."""
    occ = _map("rect_128")
    m = _pymap(rl, occ)
    ref = oracle_mod.OracleMethod(occ, "cddt", 100.0, td=108)
    w, t, bl, z = ref.cddt_table()
    # drop every third zero point: a table unlike the one built here
    keep = np.ones(len(z), bool)
    keep[::3] = False
    starts = np.concatenate([[0], np.cumsum(bl)])
    seg = np.repeat(np.arange(len(bl)), bl)
    bl2 = np.bincount(seg[keep], minlength=len(bl)).astype(np.int64)
    z2 = z[keep]
    assert starts[-1] == len(z)
    ref.load_cddt_table(w, t, bl2, z2)
    g = rl.PyCDDTCast(m, 100.0, 108)
    g.load_table(t, bl2, z2)
    q = W.free_cell_queries(occ, 5000, 8)
    out = np.empty(len(q), np.float32)
    g.calc_range_many(q, out)
    assert np.array_equal(_bits(out), _bits(ref.calc_range_many(q)))


def _pf(seed=2000, side=512, n=256, m=61, mr=200.0):
    return W.particle_filter_step(side=side, n_particles=n, n_beams=m, max_range_px=mr, seed=seed,
                                  origin=(-1.25, -2.5))


@pytest.mark.parametrize("kind", ["bl", "rm", "cddt", "pcddt"])
def test_sensor_model_and_fused_parity(rl, oracle_mod, kind):
    wl = _pf()
    m = _pymap(rl, wl.occ, wl.world)
    if kind in ("cddt", "pcddt"):
        g = rl.PyCDDTCast(m, wl.max_range, 108)
        if kind == "pcddt":
            g.prune()
    else:
        g = {"bl": rl.PyBresenhamsLine, "rm": rl.PyRayMarchingGPU}[kind](m, wl.max_range)
    ref = oracle_mod.OracleMethod(wl.occ, kind, wl.max_range, td=108, world=m.world)
    g.set_sensor_model(wl.table)
    ref.set_sensor_model(wl.table)
    if kind in ("bl", "rm"):
        _, trig = oracle_mod.world_rays(m.world, wl.ins, wl.angles)
        g.set_trig_override(trig)
    n, na = len(wl.ins), len(wl.angles)
    ranges = np.empty(n * na, np.float32)
    g.calc_range_repeat_angles(wl.ins, wl.angles, ranges)
    exp_ranges = ref.calc_range_repeat_angles(wl.ins, wl.angles)
    assert np.array_equal(_bits(ranges), _bits(exp_ranges))
    w = np.empty(n, np.float64)
    g.eval_sensor_model(wl.obs, ranges, w, na, n)
    assert np.array_equal(_bits(w), _bits(ref.eval_sensor_model(wl.obs, exp_ranges, na, n)))
    wf = np.empty(n, np.float64)
    g.calc_range_repeat_angles_eval_sensor_model(wl.ins, wl.angles, wl.obs, wf)
    assert np.array_equal(_bits(wf), _bits(ref.calc_range_repeat_angles_eval_sensor_model(wl.ins, wl.angles, wl.obs)))


@pytest.mark.parametrize("side,n,mr", [(512, 256, 200.0), (2048, 500, 1500.0)])
def test_staged_update_parity(rl, oracle_mod, side, n, mr):
    """The beam-major update with staged 8-bit windows (dt_layout 3) gives the oracle's weights bit
    for bit, for any number of particle chunks per beam -- also when the bundle's box exceeds the
    window (max range 1500 px on 2048^2), and with NaN, infinite and far-off particles."""
    wl = _pf(side=side, n=n, mr=mr)
    ins = wl.ins.copy()
    ins[0] = (np.nan, 1.0, 0.0)
    ins[1] = (1e30, -1e30, 0.5)
    ins[2] = (np.inf, 3.0, -1.0)
    ins[3, 2] = np.nan
    m = _pymap(rl, wl.occ, wl.world)
    g = rl.PyRayMarching(m, wl.max_range)
    ref = oracle_mod.OracleMethod(wl.occ, "rm", wl.max_range, world=m.world)
    g.set_sensor_model(wl.table)
    ref.set_sensor_model(wl.table)
    _, trig = oracle_mod.world_rays(m.world, ins, wl.angles)
    g.set_trig_override(trig)
    exp = ref.calc_range_repeat_angles_eval_sensor_model(ins, wl.angles, wl.obs)
    for chunks in (0, 1, 3, 40):
        g.set_schedule(3, 0, 0, chunks)
        assert g.schedule()[0] == 3 and g.schedule()[3] == chunks
        w = np.empty(len(ins), np.float64)
        g.calc_range_repeat_angles_eval_sensor_model(ins, wl.angles, wl.obs, w)
        assert np.array_equal(_bits(w), _bits(exp)), chunks
    # the per-ray entry points keep their own kernels under this schedule
    r = np.empty(len(ins) * len(wl.angles), np.float32)
    g.calc_range_repeat_angles(ins, wl.angles, r)
    assert np.array_equal(_bits(r), _bits(ref.calc_range_repeat_angles(ins, wl.angles)))


@pytest.mark.parametrize("td", [1, 72, 101])
def test_giant_lut_parity(rl, oracle_mod, td):
    """GiantLUTCast: the GPU-built table equals the oracle's; every entry point (world-frame
    queries with off-map and NaN poses, repeat angles, sensor model, fused) equals the oracle's."""
    wl = _pf(side=160, n=200, m=31, mr=80.0)
    m = _pymap(rl, wl.occ, wl.world)
    g = rl.PyGiantLUTCast(m, wl.max_range, td)
    ref = oracle_mod.OracleMethod(wl.occ, "glt", wl.max_range, td=td, world=m.world, nthreads=os.cpu_count() or 1)
    assert np.array_equal(g.lut(), ref.glt_table())
    q = wl.ins.copy()
    q[:3] = [[np.nan, 0.0, 0.0], [1e6, -1e6, 1.0], [0.0, 0.0, np.nan]]
    out = np.empty(len(q), np.float32)
    g.calc_range_many(q, out)
    assert np.array_equal(_bits(out), _bits(ref.calc_range_many(q)))
    r = np.empty(len(q) * len(wl.angles), np.float32)
    g.calc_range_repeat_angles(q, wl.angles, r)
    assert np.array_equal(_bits(r), _bits(ref.calc_range_repeat_angles(q, wl.angles)))
    g.set_sensor_model(wl.table)
    ref.set_sensor_model(wl.table)
    w = np.empty(len(q), np.float64)
    g.calc_range_repeat_angles_eval_sensor_model(q, wl.angles, wl.obs, w)
    assert np.array_equal(_bits(w), _bits(ref.calc_range_repeat_angles_eval_sensor_model(q, wl.angles, wl.obs)))


@pytest.mark.parametrize("kind", ["cddt", "pcddt"])
def test_cddt_pairs_and_radial_parity(rl, oracle_mod, kind):
    """calc_range_pair and calc_range_many_radial_optimized against the oracle on a larger map,
    host and device buffers, beam counts whose loops overlap or leave positions unwritten."""
    torch = pytest.importorskip("torch")
    wl = _pf(side=512, n=700, m=61, mr=200.0)
    m = _pymap(rl, wl.occ, wl.world)
    g = rl.PyCDDTCast(m, wl.max_range, 108)
    ref = oracle_mod.OracleMethod(wl.occ, "cddt", wl.max_range, td=108, world=m.world)
    if kind == "pcddt":
        g.prune()
        ref.prune()
    q = _queries(wl.occ, 4000, 71, spread=4.0)
    got = np.array([g.calc_range_pair(*v) for v in q[:1500]], np.float32)
    exp = np.array([ref.calc_range_pair(*v) for v in q[:1500]], np.float32)
    assert np.array_equal(_bits(got), _bits(exp))
    ins = wl.ins.copy()
    ins[:2] = [[np.nan, 0.0, 0.0], [0.0, 0.0, np.nan]]
    for nr, span in ((61, 1.5), (1081, 1.5), (100, 2.0), (8, 1.0), (2, 0.5)):
        lo, hi = float(np.float32(-span * np.pi / 2)), float(np.float32(span * np.pi / 2))
        out = np.full(len(ins) * nr, -7.0, np.float32)
        g.calc_range_many_radial_optimized(nr, lo, hi, ins, out)
        exp = np.full(len(ins) * nr, -7.0, np.float32)
        ref.calc_range_many_radial_optimized(nr, lo, hi, ins, exp)
        assert np.array_equal(_bits(out), _bits(exp)), nr
    dev = torch.device("cuda:0")
    d_out = torch.full((len(ins) * 61,), -7.0, dtype=torch.float32, device=dev)
    g.calc_range_many_radial_optimized(61, float(np.float32(-0.75 * np.pi)), float(np.float32(0.75 * np.pi)),
                                       torch.from_numpy(ins).to(dev), d_out)
    torch.cuda.synchronize()
    exp = np.full(len(ins) * 61, -7.0, np.float32)
    ref.calc_range_many_radial_optimized(61, float(np.float32(-0.75 * np.pi)), float(np.float32(0.75 * np.pi)), ins, exp)
    assert np.array_equal(_bits(d_out.cpu().numpy()), _bits(exp))


def test_fused_many_beams_underflow(rl, oracle_mod):
    """1,081 beams: products reach subnormals and zero; the in-order product stays bit-exact."""
    wl = _pf(n=64, m=1081)
    m = _pymap(rl, wl.occ, wl.world)
    g = rl.PyRayMarching(m, wl.max_range)
    ref = oracle_mod.OracleMethod(wl.occ, "rm", wl.max_range, world=m.world)
    g.set_sensor_model(wl.table)
    ref.set_sensor_model(wl.table)
    _, trig = oracle_mod.world_rays(m.world, wl.ins, wl.angles)
    g.set_trig_override(trig)
    obs = np.resize(wl.obs, len(wl.angles)).astype(np.float32)
    wf = np.empty(len(wl.ins), np.float64)
    g.calc_range_repeat_angles_eval_sensor_model(wl.ins, wl.angles, obs, wf)
    exp = ref.calc_range_repeat_angles_eval_sensor_model(wl.ins, wl.angles, obs)
    assert np.array_equal(_bits(wf), _bits(exp))


def test_fused_device_trig_weights(rl, oracle_mod):
    """Production mode (device sincosf) on the particle-filter step: weights within 1e-6 relative
    wherever every range of the particle equals the oracle's."""
    wl = _pf(n=1000)
    m = _pymap(rl, wl.occ, wl.world)
    g = rl.PyRayMarchingGPU(m, wl.max_range)
    ref = oracle_mod.OracleMethod(wl.occ, "rm", wl.max_range, world=m.world)
    g.set_sensor_model(wl.table)
    ref.set_sensor_model(wl.table)
    wf = np.empty(len(wl.ins), np.float64)
    g.calc_range_repeat_angles_eval_sensor_model(wl.ins, wl.angles, wl.obs, wf)
    exp = ref.calc_range_repeat_angles_eval_sensor_model(wl.ins, wl.angles, wl.obs)
    rel = np.abs(wf - exp) / np.maximum(np.abs(exp), 1e-300)
    assert np.mean(rel <= 1e-6) >= 0.99


def test_device_pointer_path(rl, oracle_mod):
    torch = pytest.importorskip("torch")
    wl = _pf(n=500)
    m = _pymap(rl, wl.occ, wl.world)
    g = rl.PyRayMarchingGPU(m, wl.max_range)
    g.set_sensor_model(wl.table)
    host_w = np.empty(len(wl.ins), np.float64)
    g.calc_range_repeat_angles_eval_sensor_model(wl.ins, wl.angles, wl.obs, host_w)
    dev = torch.device("cuda:0")
    ins, ang, obs = (torch.from_numpy(a).to(dev) for a in (wl.ins, wl.angles, wl.obs))
    w = torch.empty(len(wl.ins), dtype=torch.float64, device=dev)
    g.calc_range_repeat_angles_eval_sensor_model(ins, ang, obs, w)
    torch.cuda.synchronize()
    assert np.array_equal(w.cpu().numpy(), host_w)
    r = torch.empty(len(wl.ins) * len(wl.angles), dtype=torch.float32, device=dev)
    g.calc_range_repeat_angles(ins, ang, r)
    hr = np.empty(r.numel(), np.float32)
    g.calc_range_repeat_angles(wl.ins, wl.angles, hr)
    torch.cuda.synchronize()
    assert np.array_equal(r.cpu().numpy(), hr)


def test_edge_cases(rl, oracle_mod):
    occ = _map("rect_128")
    m = _pymap(rl, occ)
    g = rl.PyRayMarching(m, 50.0)
    b = rl.PyBresenhamsLine(m, 50.0)
    # empty batches
    g.calc_range_many(np.zeros((0, 3), np.float32), np.zeros(0, np.float32))
    g.set_sensor_model(W.sensor_table(51))
    w = np.full(4, -1.0)
    g.calc_range_repeat_angles_eval_sensor_model(np.zeros((4, 3), np.float32), np.zeros(0, np.float32),
                                                 np.zeros(0, np.float32), w)
    assert np.all(w == 1.0)   # empty product
    # non-finite poses return max_range, never fault
    q = np.array([[np.nan, 5, 0], [5, np.nan, 0], [5, 5, np.nan], [np.inf, 5, 0], [1e30, -1e30, 1.0],
                  [-3.0, 200.0, 2.0]], np.float32)
    for meth in (g, b):
        out = np.empty(len(q), np.float32)
        meth.calc_range_many(q, out)
        assert np.all(np.isfinite(out))
    ref = oracle_mod.OracleMethod(occ, "rm", 50.0)
    out = np.empty(len(q), np.float32)
    g.calc_range_many(q, out)
    assert np.array_equal(_bits(out), _bits(ref.calc_range_many(q)))


def test_bresenham_walk_that_skips_its_end(rl, oracle_mod):
    """A walk whose start has the fraction 1 - ulp rounds up where it crosses a power of two
    (999.99994 + 24 -> 1025.0) and never reaches its end cell 1024, so the reference's loop never
    ends.  The loop bound returns max_range and raises RLC_FLAG_BL_BOUND (1), on the GPU as in
    the oracle; a neighbouring ray that reaches its end is unaffected."""
    occ = np.zeros((64, 1100), np.uint8)
    m = _pymap(rl, occ)
    b = rl.PyBresenhamsLine(m, 23.5)
    y = float(np.float32(1000.0) - np.float32(2.0 ** -14))
    q = np.array([[5.5, y, np.pi / 2], [5.5, 999.5, np.pi / 2]], np.float32)
    trig = np.array([[np.cos(np.pi / 2), np.sin(np.pi / 2)]] * 2, np.float32)
    b.set_trig_override(trig)
    b.device_flags()   # clears
    out = np.empty(2, np.float32)
    rl._lib.call("rlc_calc_range_many", b.handle, q.ctypes.data, out.ctypes.data, 2, rl._lib.RLC_NO_WORLD, None)
    ref = oracle_mod.OracleMethod(occ, "bl", 23.5)
    exp = np.array([ref.calc_range_trig(float(a), float(bb), float(c), float(s))
                    for (a, bb, _), (c, s) in zip(q, trig)], np.float32)
    assert np.array_equal(_bits(out), _bits(exp))
    assert out[0] == np.float32(23.5) and out[1] == np.float32(23.5)
    assert b.device_flags() & 1


def test_bresenham_map_wider_than_2_pow_24(rl, oracle_mod):
    """The reference's in-grid test compares with (float)width, which rounds down for a width of
    2^24 + 1: the last column (x = 2^24) is never tested, and walks there stall (float +1 no
    longer moves them); the reference never ends them, the oracle's loop bound returns max_range.
    The GPU must agree with the oracle.  A stalled walk at 2^24 has passed the grid's in-grid
    bound min(W, (float)W) = 2^24 in its direction of motion, so the GPU ends it there without
    running into the loop bound: no RLC_FLAG_BL_BOUND."""
    w, h = (1 << 24) + 1, 2
    occ = np.zeros((w, h), np.uint8)
    occ[w - 1, :] = 1
    m = _pymap(rl, occ)
    b = rl.PyBresenhamsLine(m, 40.0)
    q = np.array([[16777190.0, 0.5, 0.0], [16777200.0, 1.5, 0.0], [16777212.0, 0.5, 0.0],
                  [16777215.0, 0.5, 0.01], [16777216.0, 0.5, np.pi], [16777100.0, 1.0, 0.02]], np.float32)
    trig = np.stack([np.cos(q[:, 2].astype(np.float64)), np.sin(q[:, 2].astype(np.float64))], 1).astype(np.float32)
    b.set_trig_override(trig)
    b.device_flags()   # clears
    out = np.empty(len(q), np.float32)
    rl._lib.call("rlc_calc_range_many", b.handle, q.ctypes.data, out.ctypes.data, len(q), rl._lib.RLC_NO_WORLD,
                 None)
    ref = oracle_mod.OracleMethod(occ, "bl", 40.0)
    exp = np.array([ref.calc_range_trig(float(x), float(y), float(c), float(s))
                    for (x, y, _), (c, s) in zip(q, trig)], np.float32)
    assert np.array_equal(_bits(out), _bits(exp))
    assert b.device_flags() & 1 == 0


def test_bresenham_walk_past_the_grid_edge_ends_there(rl, oracle_mod):
    """A walk that has left the grid in its direction of motion meets no occupied cell again, so
    the GPU ends it there with max_range (the reference walks on to its end cell and returns
    max_range too): a huge max_range costs no more than the map's size, and the results equal
    the oracle's, whose loop walks to the end.  A walk that starts off the grid and moves into it
    is not cut short."""
    occ = np.zeros((64, 48), np.uint8)
    occ[30:34, 20:24] = 1
    m = _pymap(rl, occ)
    b = rl.PyBresenhamsLine(m, 1.0e7)
    q = np.array([[10.5, 10.5, 0.0], [10.5, 10.5, np.pi / 2], [10.5, 10.5, np.pi], [10.5, 10.5, -np.pi / 2],
                  [10.5, 10.5, 0.7], [-50.5, 21.5, np.pi / 2], [31.5, -40.5, 0.0], [31.5, 90.5, np.pi],
                  [-5.0, -5.0, 0.8], [70.5, 21.5, np.pi / 2]], np.float32)
    trig = np.stack([np.cos(q[:, 2].astype(np.float64)), np.sin(q[:, 2].astype(np.float64))], 1).astype(np.float32)
    b.set_trig_override(trig)
    b.device_flags()
    out = np.empty(len(q), np.float32)
    rl._lib.call("rlc_calc_range_many", b.handle, q.ctypes.data, out.ctypes.data, len(q), rl._lib.RLC_NO_WORLD,
                 None)
    ref = oracle_mod.OracleMethod(occ, "bl", 1.0e7)
    exp = np.array([ref.calc_range_trig(float(x), float(y), float(c), float(s))
                    for (x, y, _), (c, s) in zip(q, trig)], np.float32)
    assert np.array_equal(_bits(out), _bits(exp))
    assert b.device_flags() & 1 == 0


def test_argument_errors(rl):
    occ = _map("rect_128")
    m = _pymap(rl, occ)
    g = rl.PyRayMarching(m, 50.0)
    with pytest.raises(rl._lib.RangeLibError):
        g.calc_range_repeat_angles_eval_sensor_model(np.zeros((2, 3), np.float32), np.zeros(3, np.float32),
                                                     np.zeros(3, np.float32), np.zeros(2))
    with pytest.raises(ValueError):
        g.calc_range_many(np.zeros((2, 3), np.float64), np.zeros(2, np.float32))
    g.set_sensor_model(np.ones((3, 4)))   # non-square: reference prints and returns
    with pytest.raises(rl._lib.RangeLibError):
        rl.PyCDDTCast(m, 50.0, 1)
    with pytest.raises(rl._lib.RangeLibError):   # RM schedules: prefetch 0 or 1
        g.set_schedule(0, 0, 2, 0)
    c = rl.PyCDDTCast(m, 50.0, 16)
    c.set_schedule(0, 0, 2, 0)                   # CDDT searches: 0 .. 2
    with pytest.raises(rl._lib.RangeLibError):
        c.set_schedule(0, 0, 3, 0)
    assert c.schedule()[2] == 2


def test_batch_matches_per_filter_calls(rl, oracle_mod):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda:0")
    specs = [W.FilterSpec(256, 300, 45, 120.0, 51), W.FilterSpec(512, 40, 700, 250.0, 52),
             W.FilterSpec(128, 1000, 30, 60.0, 53), W.FilterSpec(256, 7, 300, 90.0, 54),
             W.FilterSpec(128, 150, 61, 80.0, 55)]
    kinds = ["rm", "bl", "cddt", "rm", "glt"]
    filters, expect, keep = [], [], []
    for spec, kind in zip(specs, kinds):
        wl = W.batch_filter(spec)
        m = _pymap(rl, wl.occ)
        if kind == "cddt":
            g = rl.PyCDDTCast(m, wl.max_range, 108)
        elif kind == "glt":
            g = rl.PyGiantLUTCast(m, wl.max_range, 72)
        else:
            g = (rl.PyBresenhamsLine if kind == "bl" else rl.PyRayMarching)(m, wl.max_range)
        g.set_sensor_model(wl.table)
        w = np.empty(len(wl.ins), np.float64)
        g.calc_range_repeat_angles_eval_sensor_model(wl.ins, wl.angles, wl.obs, w)
        r = np.empty(len(wl.ins) * len(wl.angles), np.float32)
        g.calc_range_repeat_angles(wl.ins, wl.angles, r)
        expect.append((w, r / np.float32(1.0)))
        t = [torch.from_numpy(a).to(dev) for a in (wl.ins, wl.angles, wl.obs)]
        tw = torch.zeros(len(wl.ins), dtype=torch.float64, device=dev)
        tr = torch.zeros(len(wl.ins) * len(wl.angles), dtype=torch.float32, device=dev)
        filters.append((g, t[0], t[1], t[2], tw, tr))
        keep.append(m)
    batch = rl.PyFilterBatch(filters)
    rays, tiles = batch.info()
    assert rays == sum(len(f[1]) * len(f[2]) for f in filters) and tiles > 0
    for sched in ((0, 0, 256, 0), (1, 1, 128, 8), (2, 1, 512, 32), (2, 0, 256, 3), (4, 0, 256, 32), (5, 1, 256, 16),
                  "separate"):
        if sched == "separate":
            batch.set_product_mode(True)
            assert batch.product_mode() == "separate"
        else:
            batch.set_schedule(*sched)
        for _ in range(2):   # graph replays
            for f in filters:
                f[4].zero_()
                f[5].zero_()
            batch.run()
            torch.cuda.synchronize()
            for f, (w, r) in zip(filters, expect):
                assert np.array_equal(f[4].cpu().numpy(), w), sched
                assert np.array_equal(f[5].cpu().numpy(), r), sched
    batch.autotune()
    batch.run()
    torch.cuda.synchronize()
    for f, (w, r) in zip(filters, expect):
        assert np.array_equal(f[4].cpu().numpy(), w)


def test_batch_of_ray_marchers_schedules(rl):
    """The ray-marching-only persistent kernel: every layout and prefetch gives the per-filter weights."""
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda:0")
    filters, expect, keep = [], [], []
    for spec in (W.FilterSpec(512, 400, 61, 200.0, 61), W.FilterSpec(1024, 90, 900, 350.0, 62),
                 W.FilterSpec(256, 1200, 33, 120.0, 63)):
        wl = W.batch_filter(spec)
        m = _pymap(rl, wl.occ)
        g = rl.PyRayMarching(m, wl.max_range)
        g.set_sensor_model(wl.table)
        w = np.empty(len(wl.ins), np.float64)
        g.calc_range_repeat_angles_eval_sensor_model(wl.ins, wl.angles, wl.obs, w)
        expect.append(w)
        t = [torch.from_numpy(a).to(dev) for a in (wl.ins, wl.angles, wl.obs)]
        filters.append((g, t[0], t[1], t[2], torch.zeros(len(wl.ins), dtype=torch.float64, device=dev)))
        keep.append(m)
    batch = rl.PyFilterBatch(filters)
    for layout in (0, 1, 2, 4, 5):
        for pf in (0, 1):
            batch.set_schedule(layout, pf, 256, 16)
            batch.run()
            torch.cuda.synchronize()
            for f, w in zip(filters, expect):
                assert np.array_equal(f[4].cpu().numpy(), w), (layout, pf)


def test_batch_march_budget_edges(rl):
    """The ray-marching batch hands rays that outlast their march budget on to full warps: corridor
    maps whose wall-hugging rays march hundreds of rounds, NaN / infinite / far off-grid poses,
    max_range below one step, beam counts that fill neither a warp nor a group of four, and tiles
    of one particle give the per-filter calls' ranges and weights bit for bit, under every layout,
    prefetch, block size, tile and product mode."""
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda:0")
    rng = np.random.default_rng(77)
    cases = []
    for side, seed, n, na, mr in ((512, 31, 300, 61, 300.0), (256, 32, 41, 7, 150.0), (384, 33, 90, 129, 0.5),
                                  (200, 34, 5, 1, 220.0)):
        occ = W.corridor_map(side, seed)
        ins = W.free_cell_queries(occ, n, seed)
        if n >= 4:
            ins[0] = (np.nan, 5.0, 0.0)
            ins[1] = (5.0, 5.0, np.inf)
            ins[2] = (1e9, -1e9, 0.3)
        angles = W.laser_angles(na) if na > 1 else np.zeros(1, np.float32)
        K = int(max(mr, 1.0)) + 1
        table = W.sensor_table(K)
        obs = rng.uniform(0, mr, na).astype(np.float32)
        cases.append((occ, ins.astype(np.float32), angles.astype(np.float32), obs, table, mr))
    filters, expect, keep = [], [], []
    for occ, ins, angles, obs, table, mr in cases:
        m = _pymap(rl, occ)
        g = rl.PyRayMarching(m, mr)
        g.set_sensor_model(table)
        w = np.empty(len(ins), np.float64)
        g.calc_range_repeat_angles_eval_sensor_model(ins, angles, obs, w)
        r = np.empty(len(ins) * len(angles), np.float32)
        g.calc_range_repeat_angles(ins, angles, r)
        expect.append((w, r))
        t = [torch.from_numpy(a).to(dev) for a in (ins, angles, obs)]
        filters.append((g, t[0], t[1], t[2], torch.zeros(len(ins), dtype=torch.float64, device=dev),
                        torch.zeros(len(ins) * len(angles), dtype=torch.float32, device=dev)))
        keep.append(m)
    assert np.mean(expect[0][1] == np.float32(300.0)) < 0.9   # the corridor's rays do meet walls
    batch = rl.PyFilterBatch(filters)
    for layout in (0, 4, 5):
        for pf in (0, 1):
            for block, tile in ((32, 1), (256, 8), (512, 3)):
                for separate in (False, True):
                    batch.set_schedule(layout, pf, block, tile)
                    batch.set_product_mode(separate)
                    for f in filters:
                        f[4].fill_(-1.0)
                        f[5].fill_(-1.0)
                    batch.run()
                    torch.cuda.synchronize()
                    for f, (w, r) in zip(filters, expect):
                        key = (layout, pf, block, tile, separate)
                        assert np.array_equal(_bits(f[5].cpu().numpy()), _bits(r)), key
                        assert np.array_equal(_bits(f[4].cpu().numpy()), _bits(w)), key


def test_results_do_not_depend_on_the_schedule(rl):
    """Every schedule (DT layout x prefetch x block size x tile) gives bit-identical ranges and weights."""
    torch = pytest.importorskip("torch")
    wl = _pf(n=700, side=1024)
    m = _pymap(rl, wl.occ, wl.world)
    g = rl.PyRayMarching(m, wl.max_range)
    g.set_sensor_model(wl.table)
    base_w = np.empty(len(wl.ins), np.float64)
    base_r = np.empty(len(wl.ins) * len(wl.angles), np.float32)
    g.set_schedule(0, 256, 0, 0)
    g.calc_range_repeat_angles_eval_sensor_model(wl.ins, wl.angles, wl.obs, base_w)
    g.calc_range_repeat_angles(wl.ins, wl.angles, base_r)
    for layout in (0, 1, 2, 3, 4, 5):
        for pf in (0, 1):
            for block in (64, 128, 512):
                for tile in (0, 1, 7, 32):
                    g.set_schedule(layout, block, pf, tile)
                    w = np.empty_like(base_w)
                    r = np.empty_like(base_r)
                    g.calc_range_repeat_angles_eval_sensor_model(wl.ins, wl.angles, wl.obs, w)
                    g.calc_range_repeat_angles(wl.ins, wl.angles, r)
                    assert np.array_equal(w, base_w) and np.array_equal(r, base_r), (layout, pf, block, tile)
    dev = torch.device("cuda:0")
    ins, ang, obs = (torch.from_numpy(a).to(dev) for a in (wl.ins, wl.angles, wl.obs))
    w = torch.empty(len(wl.ins), dtype=torch.float64, device=dev)
    g.autotune(ins, ang, obs, w)
    g.calc_range_repeat_angles_eval_sensor_model(ins, ang, obs, w)
    torch.cuda.synchronize()
    assert np.array_equal(w.cpu().numpy(), base_w)


def test_host_buffers_in_place_and_staged(rl, oracle_mod):
    """Host-buffer calls give the same results whether the kernels work on the host buffers in
    place (coherent host memory access) or on staged device copies; unwritten radial positions
    keep the caller's values in both."""
    wl = _pf(n=300, m=61)
    m = _pymap(rl, wl.occ, wl.world)
    results = {}
    for mode in ("auto", "staged"):
        rl.set_host_path(mode)
        try:
            g = rl.PyRayMarching(m, wl.max_range)
            g.set_sensor_model(wl.table)
            c = rl.PyCDDTCast(m, wl.max_range, 108)
            r1 = np.empty(len(wl.ins), np.float32)
            g.calc_range_many(wl.ins, r1)
            r2 = np.empty(len(wl.ins) * len(wl.angles), np.float32)
            g.calc_range_repeat_angles(wl.ins, wl.angles, r2)
            w1 = np.empty(len(wl.ins), np.float64)
            g.eval_sensor_model(wl.obs, r2, w1, len(wl.angles), len(wl.ins))
            w2 = np.empty(len(wl.ins), np.float64)
            g.calc_range_repeat_angles_eval_sensor_model(wl.ins, wl.angles, wl.obs, w2)
            r3 = np.full(len(wl.ins) * 100, -7.0, np.float32)
            c.calc_range_many_radial_optimized(100, -3.1, 3.1, wl.ins, r3)
            results[mode] = (r1, r2, w1, w2, r3, g.calc_range(200.5, 100.5, 0.3))
        finally:
            rl.set_host_path("auto")
    for a, b in zip(results["auto"], results["staged"]):
        assert np.array_equal(np.asarray(a), np.asarray(b))
    assert (results["auto"][4] == -7.0).any()
    assert isinstance(rl.host_path_direct(), bool)


def test_cddt_json_round_trip_full_size(rl):
    """The 2048^2 rectangles-and-disks map's pruned td-108 table through serialize_json /
    from_json: the same table bit for bit and the same ranges for 1M queries."""
    wl = W.cddt_queries(side=2048, n=1_000_000, td=108, max_range=300.0)
    g = rl.PyCDDTCast(_pymap(rl, wl.occ, None), 300.0, 108)
    g.prune()
    doc = g.serialize_json()
    h = rl.PyCDDTCast.from_json(doc)
    for a, b in zip(g.table(), h.table()):
        assert np.array_equal(np.ascontiguousarray(a).view(np.uint8), np.ascontiguousarray(b).view(np.uint8))
    r1 = np.empty(len(wl.ins), np.float32)
    r2 = np.empty(len(wl.ins), np.float32)
    g.calc_range_many(wl.ins, r1)
    h.calc_range_many(wl.ins, r2)
    assert np.array_equal(_bits(r1), _bits(r2))


def test_count_steps_matches_oracle_under_every_schedule(rl, oracle_mod):
    """rlc_count_steps (the S of the roofline's algorithmic bytes) equals the oracle's march-step
    count, whatever distance-transform layout the method is scheduled with."""
    wl = _pf(n=300, side=512)
    m = _pymap(rl, wl.occ, wl.world)
    for kind in ("rm", "bl"):
        g = (rl.PyRayMarching if kind == "rm" else rl.PyBresenhamsLine)(m, wl.max_range)
        ref = oracle_mod.OracleMethod(wl.occ, kind, wl.max_range, world=m.world)
        _, trig = oracle_mod.world_rays(m.world, wl.ins, wl.angles)
        g.set_trig_override(trig)
        exp = ref.mean_steps(wl.ins, wl.angles) * len(wl.ins) * len(wl.angles)
        for layout in ((0, 1, 2, 3, 4, 5) if kind == "rm" else (0,)):
            g.set_schedule(layout, 0, 0, 0)
            assert g.count_steps(wl.ins, wl.angles) == round(exp), (kind, layout)


def test_png_map_end_to_end(rl, oracle_mod, tmp_path):
    """A map saved as PNG (OMap::save) and read back by PyOMap(path, threshold) -- the reference's
    PNG constructor -- gives the grid it was saved from, and ray marching and CDDT over it equal
    the oracle's over that grid."""
    occ = np.ascontiguousarray(W.corridor_map(512, 2024)[:400, :300])
    src = _pymap(rl, occ)
    path = str(tmp_path / "m.png")
    assert src.save(path) is False
    m = rl.PyOMap(path, 128.0)
    assert not m.error() and np.array_equal(m.occupancy, occ) and m.fn == path
    q = W.free_cell_queries(occ, 5000, 31)
    _, trig = oracle_mod.world_rays(m.world, q)
    g = rl.PyRayMarching(m, 150.0)
    g.set_trig_override(trig)
    out = np.empty(len(q), np.float32)
    g.calc_range_many(q, out)
    assert np.array_equal(_bits(out), _bits(oracle_mod.OracleMethod(occ, "rm", 150.0).calc_range_many(q)))
    c = rl.PyCDDTCast(m, 150.0, 108)
    c.calc_range_many(q, out)
    assert np.array_equal(_bits(out), _bits(oracle_mod.OracleMethod(occ, "cddt", 150.0, td=108).calc_range_many(q)))
    bad = rl.PyOMap(str(tmp_path / "missing.png"), 128.0)
    assert bad.error()


@pytest.mark.parametrize("kind", ["bl", "rm"])
def test_fused_and_batch_in_a_rotated_world(rl, oracle_mod, kind):
    """The sensor-model paths under a rotated ROS frame (world -> grid rotation, RangeLib.h:468-475):
    the fused call, the separate cast + sensor model and the batched launch equal the oracle."""
    torch = pytest.importorskip("torch")
    wl = _pf(n=600)
    m = _pymap(rl, wl.occ, (0.05, 0.45, -20.0, 15.0))
    g = (rl.PyBresenhamsLine if kind == "bl" else rl.PyRayMarching)(m, wl.max_range)
    ref = oracle_mod.OracleMethod(wl.occ, kind, wl.max_range, world=m.world)
    g.set_sensor_model(wl.table)
    ref.set_sensor_model(wl.table)
    _, trig = oracle_mod.world_rays(m.world, wl.ins, wl.angles)
    g.set_trig_override(trig)
    n, na = len(wl.ins), len(wl.angles)
    exp_w = ref.calc_range_repeat_angles_eval_sensor_model(wl.ins, wl.angles, wl.obs)
    w = np.empty(n, np.float64)
    g.calc_range_repeat_angles_eval_sensor_model(wl.ins, wl.angles, wl.obs, w)
    assert np.array_equal(_bits(w), _bits(exp_w))
    r = np.empty(n * na, np.float32)
    g.calc_range_repeat_angles(wl.ins, wl.angles, r)
    assert np.array_equal(_bits(r), _bits(ref.calc_range_repeat_angles(wl.ins, wl.angles)))
    dev = torch.device("cuda:0")
    t = [torch.from_numpy(a).to(dev) for a in (wl.ins, wl.angles, wl.obs)]
    tw = torch.zeros(n, dtype=torch.float64, device=dev)
    batch = rl.PyFilterBatch([(g, t[0], t[1], t[2], tw)])
    for separate in (False, True):
        batch.set_product_mode(separate)
        batch.run()
        torch.cuda.synchronize()
        assert np.array_equal(_bits(tw.cpu().numpy()), _bits(exp_w)), separate


def test_sensor_model_clamps_and_widest_scan(rl, oracle_mod):
    """eval_sensor_model's bin clamping (RangeLib.h:533-555) on observations and ranges below 0,
    past the table, infinite and NaN; and the fused call at the widest scan the ABI takes
    (16,384 beams per particle), both against the oracle."""
    wl = _pf(n=64)
    m = _pymap(rl, wl.occ, wl.world)
    g = rl.PyRayMarching(m, wl.max_range)
    ref = oracle_mod.OracleMethod(wl.occ, "rm", wl.max_range, world=m.world)
    g.set_sensor_model(wl.table)
    ref.set_sensor_model(wl.table)
    n, na = len(wl.ins), len(wl.angles)
    rng = np.random.default_rng(3)
    specials = np.array([-5.0, -0.0, 0.0, 1e9, np.inf, -np.inf, np.nan, 9.99, 10.0, 10.01], np.float32)
    obs = wl.obs.copy()
    obs[:len(specials)] = specials
    ranges = rng.uniform(-2.0, 15.0, n * na).astype(np.float32)
    ranges[::7] = np.resize(specials, len(ranges[::7]))
    w = np.empty(n, np.float64)
    g.eval_sensor_model(obs, ranges, w, na, n)
    assert np.array_equal(_bits(w), _bits(ref.eval_sensor_model(obs, ranges, na, n)))
    angles = np.linspace(-np.pi, np.pi, 16384, endpoint=False).astype(np.float32)
    obs_w = rng.uniform(0.0, 12.0, 16384).astype(np.float32)
    ins = wl.ins[:3]
    _, trig = oracle_mod.world_rays(m.world, ins, angles)
    g.set_trig_override(trig)
    wf = np.empty(3, np.float64)
    g.calc_range_repeat_angles_eval_sensor_model(ins, angles, obs_w, wf)
    assert np.array_equal(_bits(wf), _bits(ref.calc_range_repeat_angles_eval_sensor_model(ins, angles, obs_w)))
    with pytest.raises(rl._lib.RangeLibError):   # one beam past the limit
        g.calc_range_repeat_angles_eval_sensor_model(ins, np.zeros(16385, np.float32), np.zeros(16385, np.float32), wf)
