"""The CPU oracle against the golden vectors the reference produced (tests/golden/).

BL and RM use the recorded per-ray cosf/sinf, so these checks hold on any
IEEE host.  CDDT tables depend on the host's cosf of the slice angles; they
are compared when this host's libm reproduces the recorded slice trig.
"""
import ctypes
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden", "reference_vectors.npz")


@pytest.fixture(scope="module")
def gold():
    return dict(np.load(GOLDEN))


def _names(gold):
    return sorted({k.split("/")[0] for k in gold
                   if k.endswith("/occ") and k.count("/") == 1 and k not in ("pf/occ", "glt/occ", "basement/occ")})


def _bits(a):
    a = np.ascontiguousarray(a)
    return a.view(np.uint32 if a.dtype == np.float32 else np.uint64)


def _host_slice_trig(td):
    libm = ctypes.CDLL("libm.so.6")
    libm.cosf.restype = libm.sinf.restype = ctypes.c_float
    libm.cosf.argtypes = libm.sinf.argtypes = [ctypes.c_float]
    step = np.float32(6.28318530718 / float(np.float32(td)))
    ang = np.arange(td).astype(np.float32) * step
    return np.array([[libm.cosf(float(a)), libm.sinf(float(a))] for a in ang.astype(np.float32)], np.float32)


def test_golden_has_cases(gold):
    assert {"single_pixel", "quad", "small", "rect_96", "corridor_160x120"} <= set(_names(gold))


def test_distance_transform_and_edges(gold, oracle_mod):
    for name in _names(gold):
        occ = gold[f"{name}/occ"]
        assert np.array_equal(_bits(oracle_mod.edt(occ)), _bits(gold[f"{name}/dt"])), name
        assert np.array_equal(oracle_mod.edge_map(occ), gold[f"{name}/edge"]), name


@pytest.mark.parametrize("kind", ["bl", "rm"])
def test_bl_rm_world_frame(gold, oracle_mod, kind):
    for name in _names(gold):
        occ = gold[f"{name}/occ"]
        for wname in ("identity", "ros", "rotated"):
            key = f"{name}/{wname}"
            world = tuple(float(v) for v in gold[f"{key}/world"])
            q = gold[f"{key}/ins_any"]
            trig = gold[f"{key}/trig_any"]
            m = oracle_mod.OracleMethod(occ, kind, 60.0, world=world)
            xyh, _ = oracle_mod.world_rays(world, q)
            out = np.array([m.calc_range_trig(float(a), float(b), float(c), float(d))
                            for (a, b, _), (c, d) in zip(xyh, trig)], np.float32) * np.float32(world[0])
            assert np.array_equal(_bits(out.astype(np.float32)), _bits(gold[f"{key}/{kind}/many"])), (name, wname)


@pytest.mark.parametrize("kind", ["bl", "rm"])
def test_bl_rm_grid_frame(gold, oracle_mod, kind):
    for name in _names(gold):
        m = oracle_mod.OracleMethod(gold[f"{name}/occ"], kind, 60.0)
        q, trig = gold[f"{name}/raw/ins"], gold[f"{name}/raw/trig"]
        out = np.array([m.calc_range_trig(float(a), float(b), float(c), float(d))
                        for (a, b, _), (c, d) in zip(q, trig)], np.float32)
        assert np.array_equal(_bits(out), _bits(gold[f"{name}/raw/{kind}"])), name


@pytest.mark.parametrize("kind", ["cddt", "pcddt"])
def test_cddt_tables_and_queries(gold, oracle_mod, kind):
    if not np.array_equal(_host_slice_trig(108), gold["rect_96/slice_trig_108"]):
        pytest.skip("this host's cosf/sinf of the slice angles differ from the recorded ones")
    for name in _names(gold):
        occ = gold[f"{name}/occ"]
        m = oracle_mod.OracleMethod(occ, kind, 60.0, td=108)
        w, t, bl, z = m.cddt_table()
        assert np.array_equal(w, gold[f"{name}/{kind}_table/widths"]), name
        assert np.array_equal(_bits(t), _bits(gold[f"{name}/{kind}_table/trans"])), name
        assert np.array_equal(bl, gold[f"{name}/{kind}_table/bin_len"]), name
        assert np.array_equal(_bits(z), _bits(gold[f"{name}/{kind}_table/zeros"])), name
        assert np.array_equal(_bits(m.calc_range_many_raw(gold[f"{name}/raw/ins_in"])),
                              _bits(gold[f"{name}/raw/{kind}"])), name
        for wname in ("identity", "ros"):
            key = f"{name}/{wname}"
            world = tuple(float(v) for v in gold[f"{key}/world"])
            mw = oracle_mod.OracleMethod(occ, kind, 60.0, td=108, world=world)
            assert np.array_equal(_bits(mw.calc_range_many(gold[f"{key}/ins_in"])),
                                  _bits(gold[f"{key}/{kind}/many"])), (name, wname)


@pytest.mark.parametrize("kind", ["bl", "rm", "cddt", "pcddt"])
def test_particle_filter_step(gold, oracle_mod, kind):
    if kind in ("cddt", "pcddt") and not np.array_equal(_host_slice_trig(108), gold["pf/slice_trig_108"]):
        pytest.skip("this host's cosf/sinf of the slice angles differ from the recorded ones")
    world = tuple(float(v) for v in gold["pf/world"])
    m = oracle_mod.OracleMethod(gold["pf/occ"], kind, 100.0, td=108, world=world)
    m.set_sensor_model(gold["pf/table"])
    ins, ang, obs = gold["pf/ins"], gold["pf/angles"], gold["pf/obs"]
    n, na = len(ins), len(ang)
    r = m.calc_range_repeat_angles(ins, ang)
    assert np.array_equal(_bits(r), _bits(gold[f"pf/{kind}/ranges"]))
    assert np.array_equal(_bits(m.eval_sensor_model(obs, r, na, n)), _bits(gold[f"pf/{kind}/eval"]))
    assert np.array_equal(_bits(m.calc_range_repeat_angles_eval_sensor_model(ins, ang, obs)),
                          _bits(gold[f"pf/{kind}/fused"]))


@pytest.mark.parametrize("kind", ["cddt", "pcddt"])
def test_pairs_and_radial(gold, oracle_mod, kind):
    """calc_range_pair and calc_range_many_radial_optimized (RangeLib.h:1521-1615, 616-676)."""
    if not np.array_equal(_host_slice_trig(108), gold["pf/slice_trig_108"]):
        pytest.skip("this host's cosf/sinf of the slice angles differ from the recorded ones")
    world = tuple(float(v) for v in gold["pf/world"])
    m = oracle_mod.OracleMethod(gold["pf/occ"], kind, 100.0, td=108, world=world)
    got = np.array([m.calc_range_pair(*v) for v in gold["pair/ins"]], np.float32)
    assert np.array_equal(_bits(got), _bits(gold[f"pair/{kind}"]))
    ins = gold["pf/ins"]
    for nr in (31, 100, 7):
        lo, hi = gold[f"radial/{kind}/{nr}/span"]
        out = np.full(len(ins) * nr, -7.0, np.float32)
        m.calc_range_many_radial_optimized(nr, lo, hi, ins, out)
        assert np.array_equal(_bits(out), _bits(gold[f"radial/{kind}/{nr}"])), nr


def test_giant_lut(gold, oracle_mod):
    """GiantLUTCast table and queries (RangeLib.h:1772-1904)."""
    if not np.array_equal(_host_slice_trig(24), gold["glt/slice_trig_24"]):
        pytest.skip("this host's cosf/sinf of the angle bins differ from the recorded ones")
    m = oracle_mod.OracleMethod(gold["glt/occ"], "glt", 40.0, td=24, nthreads=4)
    assert np.array_equal(m.glt_table(), gold["glt/lut"])
    got = np.array([m.calc_range(*v) for v in gold["glt/ins"]], np.float32)
    assert np.array_equal(_bits(got), _bits(gold["glt/ranges"]))


@pytest.mark.parametrize("case", ["small/pcddt_td12", "rect/cddt_td18"])
def test_cddt_json(gold, oracle_mod, case):
    """CDDTCast::serializeJson (RangeLib.h:1690-1735): the library's serialiser over the oracle's
    table prints the reference's document byte for byte at 7 digits, and reads it back."""
    from range_libc_gb300.range_libc import cddt_json_dumps, cddt_json_loads
    name, key = case.split("/")
    td = int(key.split("_td")[1])
    if not np.array_equal(_host_slice_trig(td), gold[f"json/{name}/slice_trig_{td}"]):
        pytest.skip("this host's cosf/sinf of the slice angles differ from the recorded ones")
    ref = str(gold[f"json/{case}"])
    d = cddt_json_loads(ref)
    occ = gold[f"json/{name}/occ"]
    assert np.array_equal(d["occ"], occ) and d["theta_disc"] == td
    m = oracle_mod.OracleMethod(occ, key.split("_")[0], d["max_range"], td=td)
    w, t, bl, z = m.cddt_table()
    assert cddt_json_dumps(td, d["max_range"], t, w, bl, z, occ, d["path"], precision=7) == ref
    assert np.array_equal(d["widths"], w) and np.array_equal(d["bin_len"], bl)
    assert np.allclose(d["zeros"], z, rtol=6e-7, atol=0)   # 7 significant digits


def _table_sums(widths, trans, bin_len, zeros):
    return np.array([len(bin_len), len(zeros), float(np.sum(zeros.astype(np.float64))),
                     float(np.sum(bin_len.astype(np.float64) * np.arange(len(bin_len)))),
                     float(np.sum(trans.astype(np.float64)))], np.float64)


def test_basement_benchmark_map(gold, oracle_mod):
    """The reference's published benchmark map (basement_hallways_5cm, 1200^2, max_range 500,
    td 108) in a ROS frame: BL / RM ranges with the recorded per-ray trig; CDDT / PCDDT ranges and
    table checksums where this host's slice trig is the recorded one."""
    occ = gold["basement/occ"]
    world = tuple(float(v) for v in gold["basement/world"])
    q, trig = gold["basement/ins"], gold["basement/trig"]
    xyh, _ = oracle_mod.world_rays(world, q)
    for kind in ("bl", "rm"):
        m = oracle_mod.OracleMethod(occ, kind, 500.0, world=world)
        out = np.array([m.calc_range_trig(float(a), float(b), float(c), float(d))
                        for (a, b, _), (c, d) in zip(xyh, trig)], np.float32) * np.float32(world[0])
        assert np.array_equal(_bits(out.astype(np.float32)), _bits(gold[f"basement/{kind}/many"])), kind
    if not np.array_equal(_host_slice_trig(108), gold["basement/slice_trig_108"]):
        pytest.skip("this host's cosf/sinf of the slice angles differ from the recorded ones")
    for kind in ("cddt", "pcddt"):
        m = oracle_mod.OracleMethod(occ, kind, 500.0, td=108, world=world, nthreads=os.cpu_count() or 1)
        assert np.array_equal(_bits(m.calc_range_many(q)), _bits(gold[f"basement/{kind}/many"])), kind
        assert np.array_equal(_table_sums(*m.cddt_table()), gold[f"basement/{kind}/table_sums"]), kind
