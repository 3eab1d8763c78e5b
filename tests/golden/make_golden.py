"""Generate the golden vectors under tests/golden/ by running the reference.

Run in a checkout where the reference sources exist (RLC_REFERENCE_DIR, or
the oracle Makefile's REF): it builds the reference harness (oracle/Makefile,
target `ref`, strict IEEE flags) and records, for a set of maps, poses and
sensor tables, what the reference's own classes return:

  * OMap grids of the reference's small fixture maps, loaded by its PNG
    loader (maps/single_pixel.map.png, quad.map.png, small.map.png);
  * DistanceTransform and make_edge_map(true);
  * numpy_calc_range (world frame) and calc_range (grid frame) of
    BresenhamsLine, RayMarching, CDDTCast and pruned CDDTCast;
  * numpy_calc_range_angles, eval_sensor_model and
    calc_range_repeat_angles_eval_sensor_model on a particle-filter step;
  * CDDT tables (compressed_lut, lut_translations), unpruned and pruned;
  * CDDTCast::calc_range_pair and calc_range_many_radial_optimized on the
    particle-filter map and poses;
  * a GiantLUTCast table (giant_lut) and its calc_range queries;
  * CDDTCast::serializeJson documents (unpruned and pruned), one of them for a
    map loaded from a PNG so that its "path" field is set;
  * the reference's published benchmark map (basement_hallways_5cm, 1200^2) in a
    ROS world frame: every method's ranges and checksums of the CDDT tables.

Alongside, it stores the per-ray cosf/sinf of every BL/RM heading and the
cosf/sinf of every CDDT slice angle as this host's libm computes them, so a
consumer on another host can reproduce the reference bit for bit.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle as O  # noqa: E402
from range_libc_gb300 import workloads as W  # noqa: E402

REF = O.REF_SRC
_libm = ctypes.CDLL("libm.so.6")
_libm.cosf.restype = ctypes.c_float
_libm.cosf.argtypes = [ctypes.c_float]
_libm.sinf.restype = ctypes.c_float
_libm.sinf.argtypes = [ctypes.c_float]


def libm_trig(h: np.ndarray) -> np.ndarray:
    h = np.asarray(h, np.float32).ravel()
    return np.array([[_libm.cosf(float(v)), _libm.sinf(float(v))] for v in h], np.float32)


def slice_trig(td: int) -> np.ndarray:
    twopi_div_td = np.float32(6.28318530718 / float(np.float32(td)))
    angles = (np.arange(td, dtype=np.int64).astype(np.float32) * twopi_div_td).astype(np.float32)
    return libm_trig(angles)


def raw_heading_trig(q: np.ndarray) -> np.ndarray:
    return libm_trig(q[:, 2])


def queries(occ, n, seed, spread):
    rng = np.random.default_rng(seed)
    Wd, Hd = occ.shape
    q = np.empty((n, 3), np.float32)
    q[:, 0] = rng.uniform(-spread, Wd + spread, n)
    q[:, 1] = rng.uniform(-spread, Hd + spread, n)
    q[:, 2] = rng.uniform(-7.0, 7.0, n)
    return q


def free_queries(occ, n, seed):
    if occ.min() != 0:
        return queries(occ, n, seed, 0.0)
    q = W.free_cell_queries(occ, n, seed)
    q[:, 2] = np.random.default_rng(seed + 1).uniform(-7.0, 7.0, n)
    return q


def case_map(name, occ, out, mr, td, worlds):
    """Everything the reference computes on one map."""
    rmap = O.RefMap(occ)
    out[f"{name}/occ"] = occ
    out[f"{name}/dt"] = rmap.dt()
    out[f"{name}/edge"] = rmap.edge_map()
    out[f"{name}/slice_trig_{td}"] = slice_trig(td)
    for wname, world in worlds.items():
        wmap = O.RefMap(occ, world=world)
        s = world[0]
        # BL / RM: anywhere (also outside the map); CDDT: in-map queries (outside is undefined there)
        q_any = queries(occ, 1500, 11, spread=3.0)
        q_any[:, :2] *= s
        g_in = free_queries(occ, 1500, 12)
        q_in = g_in.copy()
        q_in[:, 0], q_in[:, 1] = W.grid_to_world(g_in[:, 0].astype(np.float64), g_in[:, 1].astype(np.float64), world)
        key = f"{name}/{wname}"
        out[f"{key}/world"] = np.array(world, np.float32)
        out[f"{key}/ins_any"] = q_any
        out[f"{key}/ins_in"] = q_in
        _, trig_any = O.world_rays(world, q_any)
        out[f"{key}/trig_any"] = trig_any
        for kind in ("bl", "rm"):
            m = O.RefMethod(wmap, kind, mr)
            out[f"{key}/{kind}/many"] = m.calc_range_many(q_any)
        if world[1] == 0.0:
            for kind in ("cddt", "pcddt"):
                m = O.RefMethod(wmap, kind, mr, td)
                out[f"{key}/{kind}/many"] = m.calc_range_many(q_in)
    # grid-frame calc_range (no transform)
    q_raw = queries(occ, 1000, 13, spread=2.0)
    out[f"{name}/raw/ins"] = q_raw
    out[f"{name}/raw/trig"] = raw_heading_trig(q_raw)
    for kind in ("bl", "rm"):
        m = O.RefMethod(rmap, kind, mr)
        out[f"{name}/raw/{kind}"] = m.calc_range_many_raw(q_raw)
    q_raw_in = free_queries(occ, 1000, 14)
    out[f"{name}/raw/ins_in"] = q_raw_in
    for kind in ("cddt", "pcddt"):
        m = O.RefMethod(rmap, kind, mr, td)
        out[f"{name}/raw/{kind}"] = m.calc_range_many_raw(q_raw_in)
        widths, trans, bin_len, zeros = m.cddt_table()
        out[f"{name}/{kind}_table/widths"] = widths
        out[f"{name}/{kind}_table/trans"] = trans
        out[f"{name}/{kind}_table/bin_len"] = bin_len
        out[f"{name}/{kind}_table/zeros"] = zeros


def case_particle_filter(out):
    wl = W.particle_filter_step(side=256, n_particles=200, n_beams=31, max_range_px=100.0, seed=9,
                                origin=(-1.5, -0.75))
    world = tuple(float(np.float32(v)) for v in wl.world)
    rmap = O.RefMap(wl.occ, world=world)
    out["pf/occ"] = wl.occ
    out["pf/world"] = np.array(world, np.float32)
    out["pf/ins"] = wl.ins
    out["pf/angles"] = wl.angles
    out["pf/obs"] = wl.obs
    out["pf/table"] = wl.table
    _, trig = O.world_rays(world, wl.ins, wl.angles)
    out["pf/trig"] = trig
    out["pf/slice_trig_108"] = slice_trig(108)
    n, na = len(wl.ins), len(wl.angles)
    for kind in ("bl", "rm", "cddt", "pcddt"):
        m = O.RefMethod(rmap, kind, wl.max_range, 108)
        m.set_sensor_model(wl.table)
        r = m.calc_range_repeat_angles(wl.ins, wl.angles)
        out[f"pf/{kind}/ranges"] = r
        out[f"pf/{kind}/eval"] = m.eval_sensor_model(wl.obs, r, na, n)
        out[f"pf/{kind}/fused"] = m.calc_range_repeat_angles_eval_sensor_model(wl.ins, wl.angles, wl.obs)


def case_pairs_radial_glt(out):
    wl = W.particle_filter_step(side=256, n_particles=200, n_beams=31, max_range_px=100.0, seed=9,
                                origin=(-1.5, -0.75))
    world = tuple(float(np.float32(v)) for v in wl.world)
    rmap = O.RefMap(wl.occ, world=world)
    rng = np.random.default_rng(404)
    q = np.stack([rng.uniform(0, 255.99, 3000), rng.uniform(0, 255.99, 3000), rng.uniform(-9, 9, 3000)], 1)
    q = q.astype(np.float32)
    q[:300, :2] = np.floor(q[:300, :2]) + 0.5
    out["pair/ins"] = q
    for kind in ("cddt", "pcddt"):
        m = O.RefMethod(rmap, kind, wl.max_range, 108)
        out[f"pair/{kind}"] = np.array([m.calc_range_pair(*v) for v in q], np.float32)
        for nr, span in ((31, 1.5), (100, 2.0), (7, 2.0)):
            lo, hi = np.float32(-span * np.pi / 2), np.float32(span * np.pi / 2)
            o = np.full(len(wl.ins) * nr + 4 * nr, -7.0, np.float32)
            m.calc_range_many_radial_optimized(nr, lo, hi, wl.ins, o)
            out[f"radial/{kind}/{nr}"] = o[: len(wl.ins) * nr]
            out[f"radial/{kind}/{nr}/span"] = np.array([lo, hi], np.float32)
    occ = np.ascontiguousarray(W.rect_disk_map(96, 101)[:64, :48])
    g = O.RefMethod(O.RefMap(occ), "glt", 40.0, 24)
    out["glt/occ"] = occ
    out["glt/slice_trig_24"] = slice_trig(24)
    out["glt/lut"] = g.glt_table()
    qg = np.stack([rng.uniform(-2, 66, 2000), rng.uniform(-2, 50, 2000), rng.uniform(-20, 20, 2000)], 1)
    qg = qg.astype(np.float32)
    out["glt/ins"] = qg
    out["glt/ranges"] = np.array([g.calc_range(*v) for v in qg], np.float32)


def _table_sums(m):
    widths, trans, bin_len, zeros = m.cddt_table()
    return np.array([len(bin_len), len(zeros), float(np.sum(zeros.astype(np.float64))),
                     float(np.sum(bin_len.astype(np.float64) * np.arange(len(bin_len)))),
                     float(np.sum(trans.astype(np.float64)))], np.float64)


def case_basement(out):
    """The reference's published benchmark map (maps/basement_hallways_5cm.png, 1200^2, max_range
    500 px, theta_discretization 108 as in its main.cpp) in a ROS world frame at 0.05 m/px: ranges
    of every method for free-cell queries, and checksums of the CDDT / PCDDT tables."""
    rm_ = O.RefMap(png=os.path.join(REF, "maps", "basement_hallways_5cm.png"), threshold=128.0)
    occ = rm_.occ
    world = O.world_tuple(0.05, 0.0, -30.0, -20.0)
    wmap = O.RefMap(occ, world=world)
    g = free_queries(occ, 4000, 71)
    q = g.copy()
    q[:, 0], q[:, 1] = W.grid_to_world(g[:, 0].astype(np.float64), g[:, 1].astype(np.float64), world)
    _, trig = O.world_rays(world, q)
    out["basement/occ"] = occ
    out["basement/world"] = np.array(world, np.float32)
    out["basement/ins"] = q
    out["basement/trig"] = trig
    out["basement/slice_trig_108"] = slice_trig(108)
    for kind in ("bl", "rm", "cddt", "pcddt"):
        m = O.RefMethod(wmap, kind, 500.0, 108)
        out[f"basement/{kind}/many"] = m.calc_range_many(q)
        if kind in ("cddt", "pcddt"):
            out[f"basement/{kind}/table_sums"] = _table_sums(m)


def case_json(out):
    here = os.getcwd()
    os.chdir(os.path.join(REF, "maps"))   # the document records the PNG path as given
    try:
        pm = O.RefMap(png="small.map.png", threshold=128.0)
    finally:
        os.chdir(here)
    out["json/small/occ"] = pm.occ
    out["json/small/slice_trig_12"] = slice_trig(12)
    out["json/small/pcddt_td12"] = np.array(_pruned(O.RefMethod(pm, "cddt", 30.0, 12)).cddt_json())
    occ = np.ascontiguousarray(W.rect_disk_map(96, 101)[:40, :56])
    out["json/rect/occ"] = occ
    out["json/rect/slice_trig_18"] = slice_trig(18)
    out["json/rect/cddt_td18"] = np.array(O.RefMethod(O.RefMap(occ), "cddt", 25.0, 18).cddt_json())


def _pruned(m):
    m.prune()
    return m


def main():
    O.build(reference=True)
    out = {}
    maps = {}
    for f in ("single_pixel.map.png", "quad.map.png", "small.map.png"):
        rm_ = O.RefMap(png=os.path.join(REF, "maps", f), threshold=128.0)
        maps[f.split(".")[0]] = rm_.occ
    maps["rect_96"] = W.rect_disk_map(96, 101)
    maps["corridor_160x120"] = np.ascontiguousarray(W.corridor_map(256, 102)[:160, :120])
    worlds = {
        "identity": O.world_tuple(),
        "ros": O.world_tuple(0.05, 0.0, -1.25, -0.5),
        "rotated": O.world_tuple(0.1, 0.6, 1.0, -2.0),
    }
    for name, occ in maps.items():
        case_map(name, occ, out, mr=60.0, td=108, worlds=worlds)
    case_particle_filter(out)
    case_pairs_radial_glt(out)
    case_json(out)
    case_basement(out)
    path = os.path.join(HERE, "reference_vectors.npz")
    np.savez_compressed(path, **out)
    print(f"wrote {path}: {len(out)} arrays, {os.path.getsize(path) / 1e6:.2f} MB")


if __name__ == "__main__":
    main()
