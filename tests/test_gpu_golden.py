"""The CUDA library against the golden vectors the reference produced.

The reference was run on another host; its per-ray cosf/sinf (BL, RM) and
its slice cosf/sinf (CDDT) are part of the vectors and are handed to the
library (trig override, CDDT trig tables) so that every comparison is
bit-exact on any host.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_vectors.npz")


@pytest.fixture(scope="module")
def gold():
    return dict(np.load(GOLDEN))


def _names(gold):
    return sorted({k.split("/")[0] for k in gold
                   if k.endswith("/occ") and k.count("/") == 1 and k not in ("pf/occ", "glt/occ", "basement/occ")})


def _bits(a):
    a = np.ascontiguousarray(a)
    return a.view(np.uint32 if a.dtype == np.float32 else np.uint64)


def _map(rl, occ, world=None):
    m = rl.PyOMap(np.ascontiguousarray(occ.T))
    if world is not None:
        m.set_world(*[float(v) for v in world[:4]], sin_angle=float(world[4]), cos_angle=float(world[5]))
    return m


def test_distance_transform_and_edges(rl, gold):
    for name in _names(gold):
        occ = gold[f"{name}/occ"]
        m = _map(rl, occ)
        dt = np.empty(occ.shape, np.float32)
        rl._lib.call("rlc_map_distance_transform", m.handle, dt.ctypes.data_as(rl._lib._f32p))
        assert np.array_equal(_bits(dt), _bits(gold[f"{name}/dt"])), name
        e = np.empty(occ.shape, np.uint8)
        rl._lib.call("rlc_map_edge_map", m.handle, e.ctypes.data_as(rl._lib._u8p))
        assert np.array_equal(e, gold[f"{name}/edge"]), name


@pytest.mark.parametrize("kind", ["bl", "rm"])
def test_bl_rm(rl, gold, kind):
    cls = rl.PyBresenhamsLine if kind == "bl" else rl.PyRayMarching
    for name in _names(gold):
        occ = gold[f"{name}/occ"]
        for wname in ("identity", "ros", "rotated"):
            key = f"{name}/{wname}"
            g = cls(_map(rl, occ, gold[f"{key}/world"]), 60.0)
            g.set_trig_override(gold[f"{key}/trig_any"])
            q = gold[f"{key}/ins_any"]
            out = np.empty(len(q), np.float32)
            g.calc_range_many(q, out)
            assert np.array_equal(_bits(out), _bits(gold[f"{key}/{kind}/many"])), (name, wname)
        g = cls(_map(rl, occ), 60.0)
        g.set_trig_override(gold[f"{name}/raw/trig"])
        q = gold[f"{name}/raw/ins"]
        out = np.empty(len(q), np.float32)
        rl._lib.call("rlc_calc_range_many", g.handle, q.ctypes.data, out.ctypes.data, len(q),
                     rl._lib.RLC_NO_WORLD, None)
        assert np.array_equal(_bits(out), _bits(gold[f"{name}/raw/{kind}"])), name


@pytest.mark.parametrize("kind", ["cddt", "pcddt"])
def test_cddt(rl, gold, kind):
    for name in _names(gold):
        occ = gold[f"{name}/occ"]
        trig = gold[f"{name}/slice_trig_108"]
        for wname in ("identity", "ros"):
            key = f"{name}/{wname}"
            g = rl.PyCDDTCast(_map(rl, occ, gold[f"{key}/world"]), 60.0, 108, trig=(trig[:, 0], trig[:, 1]))
            if kind == "pcddt":
                g.prune()
            w, t, bl, z = g.table()
            assert np.array_equal(w, gold[f"{name}/{kind}_table/widths"]), name
            assert np.array_equal(_bits(t), _bits(gold[f"{name}/{kind}_table/trans"])), name
            assert np.array_equal(bl, gold[f"{name}/{kind}_table/bin_len"]), name
            assert np.array_equal(_bits(z), _bits(gold[f"{name}/{kind}_table/zeros"])), name
            q = gold[f"{key}/ins_in"]
            out = np.empty(len(q), np.float32)
            g.calc_range_many(q, out)
            assert np.array_equal(_bits(out), _bits(gold[f"{key}/{kind}/many"])), (name, wname)
            if wname == "identity":
                qr = gold[f"{name}/raw/ins_in"]
                o2 = np.empty(len(qr), np.float32)
                rl._lib.call("rlc_calc_range_many", g.handle, qr.ctypes.data, o2.ctypes.data, len(qr),
                             rl._lib.RLC_NO_WORLD, None)
                assert np.array_equal(_bits(o2), _bits(gold[f"{name}/raw/{kind}"])), name


@pytest.mark.parametrize("kind", ["bl", "rm", "cddt", "pcddt"])
def test_particle_filter_step(rl, gold, kind):
    world = gold["pf/world"]
    m = _map(rl, gold["pf/occ"], world)
    if kind in ("cddt", "pcddt"):
        trig = gold["pf/slice_trig_108"]
        g = rl.PyCDDTCast(m, 100.0, 108, trig=(trig[:, 0], trig[:, 1]))
        if kind == "pcddt":
            g.prune()
    else:
        g = (rl.PyBresenhamsLine if kind == "bl" else rl.PyRayMarchingGPU)(m, 100.0)
        g.set_trig_override(gold["pf/trig"])
    g.set_sensor_model(gold["pf/table"])
    ins, ang, obs = gold["pf/ins"], gold["pf/angles"], gold["pf/obs"]
    n, na = len(ins), len(ang)
    r = np.empty(n * na, np.float32)
    g.calc_range_repeat_angles(ins, ang, r)
    assert np.array_equal(_bits(r), _bits(gold[f"pf/{kind}/ranges"]))
    w = np.empty(n, np.float64)
    g.eval_sensor_model(obs, r, w, na, n)
    assert np.array_equal(_bits(w), _bits(gold[f"pf/{kind}/eval"]))
    g.calc_range_repeat_angles_eval_sensor_model(ins, ang, obs, w)
    assert np.array_equal(_bits(w), _bits(gold[f"pf/{kind}/fused"]))


@pytest.mark.parametrize("kind", ["cddt", "pcddt"])
def test_pairs_and_radial(rl, gold, kind):
    """CDDTCast::calc_range_pair and calc_range_many_radial_optimized against the reference's vectors."""
    trig = gold["pf/slice_trig_108"]
    g = rl.PyCDDTCast(_map(rl, gold["pf/occ"], gold["pf/world"]), 100.0, 108, trig=(trig[:, 0], trig[:, 1]))
    if kind == "pcddt":
        g.prune()
    got = np.array([g.calc_range_pair(*v) for v in gold["pair/ins"]], np.float32)
    assert np.array_equal(_bits(got), _bits(gold[f"pair/{kind}"]))
    ins = gold["pf/ins"]
    for nr in (31, 100, 7):
        lo, hi = gold[f"radial/{kind}/{nr}/span"]
        out = np.full(len(ins) * nr, -7.0, np.float32)
        g.calc_range_many_radial_optimized(nr, float(lo), float(hi), ins, out)
        assert np.array_equal(_bits(out), _bits(gold[f"radial/{kind}/{nr}"])), nr


def test_giant_lut(rl, gold):
    """GiantLUTCast: the GPU-built table and its queries against the reference's."""
    t = gold["glt/slice_trig_24"]
    g = rl.PyGiantLUTCast(_map(rl, gold["glt/occ"]), 40.0, 24, trig=(t[:, 0], t[:, 1]))
    assert np.array_equal(g.lut(), gold["glt/lut"])
    q = np.ascontiguousarray(gold["glt/ins"])
    out = np.empty(len(q), np.float32)
    rl._lib.call("rlc_calc_range_many", g.handle, q.ctypes.data, out.ctypes.data, len(q), rl._lib.RLC_NO_WORLD, None)
    assert np.array_equal(_bits(out), _bits(gold["glt/ranges"]))


@pytest.mark.parametrize("case", ["small/pcddt_td12", "rect/cddt_td18"])
def test_cddt_json(rl, gold, case):
    """serializeJson of the GPU-built table is the reference's document (7 digits); at 9 digits
    it restores the table exactly, through load_json and through from_json."""
    name, key = case.split("/")
    td = int(key.split("_td")[1])
    trig = gold[f"json/{name}/slice_trig_{td}"]
    ref = str(gold[f"json/{case}"])
    occ = gold[f"json/{name}/occ"]
    m = _map(rl, occ)
    m.fn = "small.map.png" if name == "small" else ""
    g = rl.PyCDDTCast(m, 30.0 if name == "small" else 25.0, td, trig=(trig[:, 0], trig[:, 1]))
    if key.startswith("pcddt"):
        g.prune()
    assert g.serialize_json(precision=7) == ref
    doc = g.serialize_json()
    w, t, bl, z = g.table()
    h = rl.PyCDDTCast.from_json(doc, trig=(trig[:, 0], trig[:, 1]))
    w2, t2, bl2, z2 = h.table()
    assert np.array_equal(w2, w) and np.array_equal(bl2, bl)
    assert np.array_equal(_bits(t2), _bits(t)) and np.array_equal(_bits(z2), _bits(z))
    assert h.serialize_json() == doc
    u = rl.PyCDDTCast(_map(rl, occ), 25.0, td, trig=(trig[:, 0], trig[:, 1]))
    u.load_json(ref)   # the reference's 7-digit document
    assert np.array_equal(u.table()[2], bl)
    assert np.allclose(u.table()[3], z, rtol=6e-7, atol=0)
    with pytest.raises(ValueError):
        rl.PyCDDTCast(_map(rl, occ), 25.0, td + 1).load_json(ref)


def test_basement_benchmark_map(rl, gold):
    """The reference's published benchmark map (basement_hallways_5cm, 1200^2, max_range 500,
    td 108) in a ROS frame: every method's ranges and the CDDT / PCDDT table checksums."""
    occ, world = gold["basement/occ"], gold["basement/world"]
    q = gold["basement/ins"]
    for kind, cls in (("bl", rl.PyBresenhamsLine), ("rm", rl.PyRayMarching)):
        g = cls(_map(rl, occ, world), 500.0)
        g.set_trig_override(gold["basement/trig"])
        out = np.empty(len(q), np.float32)
        g.calc_range_many(q, out)
        assert np.array_equal(_bits(out), _bits(gold[f"basement/{kind}/many"])), kind
    t = gold["basement/slice_trig_108"]
    for kind in ("cddt", "pcddt"):
        g = rl.PyCDDTCast(_map(rl, occ, world), 500.0, 108, trig=(t[:, 0], t[:, 1]))
        if kind == "pcddt":
            g.prune()
        for search in (0, 2):
            g.set_schedule(0, 0, search, 0)
            out = np.empty(len(q), np.float32)
            g.calc_range_many(q, out)
            assert np.array_equal(_bits(out), _bits(gold[f"basement/{kind}/many"])), (kind, search)
        w, tr, bl, z = g.table()
        sums = np.array([len(bl), len(z), float(np.sum(z.astype(np.float64))),
                         float(np.sum(bl.astype(np.float64) * np.arange(len(bl)))),
                         float(np.sum(tr.astype(np.float64)))], np.float64)
        assert np.array_equal(sums, gold[f"basement/{kind}/table_sums"]), kind
