"""The CPU oracle against the reference itself, compiled from its sources (oracle/_ref).

Runs only where the reference sources are present (the harness cannot be
built elsewhere).  Larger and more varied than the golden vectors: several
maps and world frames, every method, sensor tables up to K = 201 and beams
up to 1,081 (weights reach subnormals and zero).
"""
import numpy as np
import pytest

from range_libc_gb300 import workloads as W


@pytest.fixture(scope="module")
def O():
    import oracle
    if not oracle.ref_available():
        try:
            oracle.build(reference=True)
        except Exception as e:  # noqa: BLE001
            pytest.skip(f"reference harness unavailable: {e}")
    if not oracle.ref_available():
        pytest.skip("reference sources not present")
    return oracle


def _bits(a):
    a = np.ascontiguousarray(a)
    return a.view(np.uint32 if a.dtype == np.float32 else np.uint64)


MAPS = {
    "rect_512": lambda: W.rect_disk_map(512, 1000),
    "corridor_384x256": lambda: np.ascontiguousarray(W.corridor_map(512, 2000)[:384, :256]),
    "rect_2048": lambda: W.rect_disk_map(2048, 3000),
}


@pytest.mark.parametrize("name", list(MAPS))
def test_distance_transform(O, name):
    occ = MAPS[name]()
    assert np.array_equal(_bits(O.edt(occ)), _bits(O.RefMap(occ).dt()))


@pytest.mark.parametrize("kind", ["bl", "rm", "cddt", "pcddt"])
@pytest.mark.parametrize("world", [(1.0, 0.0, 0.0, 0.0), (0.05, 0.0, -12.5, -7.5), (0.07, 1.1, 3.0, 2.0)])
def test_queries(O, kind, world):
    occ = MAPS["rect_512"]()
    w = O.world_tuple(*world)
    q = W.free_cell_queries(occ, 20000, 5)
    q[:, 0], q[:, 1] = W.grid_to_world(q[:, 0].astype(np.float64), q[:, 1].astype(np.float64), w)
    if kind in ("cddt", "pcddt") and world[1] != 0.0:
        pytest.skip("rotated worlds land CDDT queries off the map (undefined in the reference)")
    ref = O.RefMethod(O.RefMap(occ, world=w), kind, 300.0, 108)
    orc = O.OracleMethod(occ, kind, 300.0, td=108, world=w)
    assert np.array_equal(_bits(orc.calc_range_many(q)), _bits(ref.calc_range_many(q)))
    if kind in ("bl", "rm"):
        rng = np.random.default_rng(8)
        qa = np.stack([rng.uniform(-20, 530, 5000) * world[0], rng.uniform(-20, 530, 5000) * world[0],
                       rng.uniform(-20, 20, 5000)], 1).astype(np.float32)
        assert np.array_equal(_bits(orc.calc_range_many(qa)), _bits(ref.calc_range_many(qa)))


@pytest.mark.parametrize("td", [108, 216, 37])
def test_cddt_tables(O, td):
    occ = MAPS["corridor_384x256"]()
    for kind in ("cddt", "pcddt"):
        ref = O.RefMethod(O.RefMap(occ), kind, 200.0, td)
        orc = O.OracleMethod(occ, kind, 200.0, td=td)
        for a, b in zip(orc.cddt_table(), ref.cddt_table()):
            assert np.array_equal(_bits(a) if a.dtype == np.float32 else a, _bits(b) if b.dtype == np.float32 else b)


@pytest.mark.parametrize("kind", ["rm", "bl", "cddt"])
@pytest.mark.parametrize("beams", [61, 1081])
def test_sensor_model_paths(O, kind, beams):
    wl = W.particle_filter_step(side=512, n_particles=300, n_beams=beams, max_range_px=200.0, seed=44)
    w = tuple(float(np.float32(v)) for v in wl.world)
    ref = O.RefMethod(O.RefMap(wl.occ, world=w), kind, 200.0, 108)
    orc = O.OracleMethod(wl.occ, kind, 200.0, td=108, world=w)
    ref.set_sensor_model(wl.table)
    orc.set_sensor_model(wl.table)
    obs = np.resize(wl.obs, beams).astype(np.float32)
    n, na = len(wl.ins), len(wl.angles)
    r_ref = ref.calc_range_repeat_angles(wl.ins, wl.angles)
    assert np.array_equal(_bits(orc.calc_range_repeat_angles(wl.ins, wl.angles)), _bits(r_ref))
    assert np.array_equal(_bits(orc.eval_sensor_model(obs, r_ref, na, n)),
                          _bits(ref.eval_sensor_model(obs, r_ref, na, n)))
    wf = ref.calc_range_repeat_angles_eval_sensor_model(wl.ins, wl.angles, obs)
    assert np.array_equal(_bits(orc.calc_range_repeat_angles_eval_sensor_model(wl.ins, wl.angles, obs)), _bits(wf))
    if beams == 1081:
        assert np.any(wf == 0.0) or np.any(wf < 2.3e-308)   # underflow is exercised


def test_multithreaded_oracle_equals_single(O):
    wl = W.particle_filter_step(side=512, n_particles=500, n_beams=61, max_range_px=200.0, seed=45)
    w = tuple(float(np.float32(v)) for v in wl.world)
    orc = O.OracleMethod(wl.occ, "rm", 200.0, world=w)
    orc.set_sensor_model(wl.table)
    a = orc.calc_range_repeat_angles_eval_sensor_model(wl.ins, wl.angles, wl.obs, nthreads=1)
    b = orc.calc_range_repeat_angles_eval_sensor_model(wl.ins, wl.angles, wl.obs, nthreads=7)
    assert np.array_equal(a, b)


@pytest.mark.parametrize("td", [36, 101])
def test_giant_lut(O, td):
    """GiantLUTCast: the 16-bit table and its queries (RangeLib.h:1772-1904)."""
    occ = np.ascontiguousarray(W.rect_disk_map(128, 21)[:128, :96])
    orc = O.OracleMethod(occ, "glt", 60.0, td=td, nthreads=4)
    ref = O.RefMethod(O.RefMap(occ), "glt", 60.0, td)
    assert np.array_equal(orc.glt_table(), ref.glt_table())
    rng = np.random.default_rng(td)
    q = np.stack([rng.uniform(-3, 131, 4000), rng.uniform(-3, 99, 4000), rng.uniform(-30, 30, 4000)], 1)
    q = q.astype(np.float32)
    q[:5] = [[np.nan, 1, 1], [1, np.nan, 1], [1, 1, np.nan], [127.99, 95.99, 0], [128, 0, 0]]
    got = np.array([orc.calc_range(*v) for v in q[5:]], np.float32)
    exp = np.array([ref.calc_range(*v) for v in q[5:]], np.float32)
    assert np.array_equal(_bits(got), _bits(exp))


def test_cddt_calc_range_pair(O):
    """calc_range_pair (RangeLib.h:1521-1615) on free, occupied and on-zero-point queries."""
    occ = MAPS["rect_512"]()
    for kind in ("cddt", "pcddt"):
        orc = O.OracleMethod(occ, kind, 300.0, td=108)
        ref = O.RefMethod(O.RefMap(occ), kind, 300.0, 108)
        rng = np.random.default_rng(3)
        q = np.stack([rng.uniform(0, 511.99, 20000), rng.uniform(0, 511.99, 20000),
                      rng.uniform(-12, 12, 20000)], 1).astype(np.float32)
        q[:2000, :2] = np.floor(q[:2000, :2]) + 0.5      # cell centres, some occupied
        got = np.array([orc.calc_range_pair(*v) for v in q], np.float32)
        exp = np.array([ref.calc_range_pair(*v) for v in q], np.float32)
        assert np.array_equal(_bits(got), _bits(exp)), kind


@pytest.mark.parametrize("num_rays,span", [(61, 1.5), (1081, 1.5), (100, 2.0), (10, 1.0), (7, 2.0), (3, 0.6), (2, 1.0)])
def test_cddt_radial(O, num_rays, span):
    """calc_range_many_radial_optimized (RangeLib.h:616-676) on the particle-filter workload's poses,
    including beam counts whose pairs overlap the single casts or leave positions unwritten."""
    wl = W.particle_filter_step(side=512, n_particles=300, n_beams=61, max_range_px=200.0, origin=(-1.25, -2.5))
    w = O.world_tuple(*wl.world[:4])
    orc = O.OracleMethod(wl.occ, "cddt", wl.max_range, td=108, world=w)
    ref = O.RefMethod(O.RefMap(wl.occ, world=w), "cddt", wl.max_range, 108)
    lo, hi = np.float32(-span * np.pi / 2), np.float32(span * np.pi / 2)
    n = len(wl.ins)
    o_ref = np.full(n * num_rays + 4 * num_rays, -7.0, np.float32)   # room for the reference's row overrun
    o_orc = np.full(n * num_rays, -7.0, np.float32)
    ref.calc_range_many_radial_optimized(num_rays, lo, hi, wl.ins, o_ref)
    orc.calc_range_many_radial_optimized(num_rays, lo, hi, wl.ins, o_orc)
    assert np.array_equal(_bits(o_orc), _bits(o_ref[: n * num_rays]))


@pytest.mark.parametrize("kind,td", [("cddt", 108), ("pcddt", 108), ("pcddt", 7)])
def test_cddt_json(O, kind, td):
    """serializeJson: the library's serialiser prints the reference's document byte for byte at 7
    significant digits; at 9 its document reads back to the table bit for bit."""
    from range_libc_gb300.range_libc import cddt_json_dumps, cddt_json_loads
    occ = np.ascontiguousarray(MAPS["corridor_384x256"]()[:200, :150])
    ref = O.RefMethod(O.RefMap(occ), "cddt", 120.0, td)
    orc = O.OracleMethod(occ, kind, 120.0, td=td)
    if kind == "pcddt":
        ref.prune()
    w, t, bl, z = orc.cddt_table()
    assert cddt_json_dumps(td, 120.0, t, w, bl, z, occ, "", precision=7) == ref.cddt_json()
    d = cddt_json_loads(cddt_json_dumps(td, 120.0, t, w, bl, z, occ))
    for k, v in (("trans", t), ("widths", w), ("bin_len", bl), ("zeros", z), ("occ", occ)):
        assert np.array_equal(_bits(d[k]) if k in ("trans", "zeros") else d[k],
                              _bits(v) if k in ("trans", "zeros") else v), k


def test_png_maps_match_reference_loader(O, tmp_path):
    """The library's PNG decoder against the reference's OMap(filename, 128) on every map the
    reference ships (1x1 to 10976x10976; grey 1/8-bit, RGB, RGBA), and the reference's loader on
    a map saved by rlc_png_save_occupancy."""
    import os
    from range_libc_gb300 import _lib
    from range_libc_gb300.range_libc import png_occupancy
    maps = os.path.join(O.REF_SRC, "maps")
    names = sorted(f for f in os.listdir(maps) if f.endswith(".png"))
    assert len(names) >= 10
    for f in names:
        assert np.array_equal(png_occupancy(os.path.join(maps, f)), O.RefMap(png=os.path.join(maps, f)).occ), f
    occ = np.ascontiguousarray(MAPS["corridor_384x256"]())
    path = str(tmp_path / "saved.png")
    assert _lib.lib().rlc_png_save_occupancy(path.encode(), occ.ctypes.data, occ.shape[0], occ.shape[1]) == 0
    assert np.array_equal(O.RefMap(png=path).occ, occ)


@pytest.mark.parametrize("case", ["all_free", "all_walls", "one_cell", "td1", "td2"])
def test_cddt_json_edge_cases(O, case):
    """serializeJson's document on degenerate tables: no zero points at all, a map of walls only,
    a 1x1 map, one and two angle slices -- byte for byte at 7 digits, exact round trip at 9."""
    from range_libc_gb300.range_libc import cddt_json_dumps, cddt_json_loads
    occ = {"all_free": np.zeros((20, 14), np.uint8), "all_walls": np.ones((9, 11), np.uint8),
           "one_cell": np.zeros((1, 1), np.uint8)}.get(case, MAPS["corridor_384x256"]()[:60, :40].copy())
    td = {"td1": 1, "td2": 2}.get(case, 12)
    ref = O.RefMethod(O.RefMap(np.ascontiguousarray(occ)), "cddt", 30.0, td)
    orc = O.OracleMethod(occ, "cddt", 30.0, td=td)
    w, t, bl, z = orc.cddt_table()
    assert cddt_json_dumps(td, 30.0, t, w, bl, z, occ, "", precision=7) == ref.cddt_json()
    d = cddt_json_loads(cddt_json_dumps(td, 30.0, t, w, bl, z, occ))
    assert np.array_equal(d["bin_len"], bl) and np.array_equal(_bits(d["zeros"]), _bits(z))
    assert np.array_equal(d["occ"], occ) and d["theta_disc"] == td
