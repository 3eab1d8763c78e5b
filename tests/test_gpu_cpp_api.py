"""A C++ caller of the reference's ranges:: API (include/RangeLib.h) against the oracle.

Compiles tests/cpp/shim_caller.cpp with g++ against include/ and the built
library, runs it on a seeded map, and compares every output with the oracle.
The device's own sincosf is used, so BL and RM ranges may differ on rare rays
(a last-bit cos/sin difference moving a ray across a cell corner).
"""
import os
import subprocess

import numpy as np
import pytest

from range_libc_gb300 import workloads as W
from range_libc_gb300.range_libc import cddt_json_dumps

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_cpp_caller(rl, oracle_mod, tmp_path):
    lib = rl.library_path()
    exe = tmp_path / "shim_caller"
    subprocess.check_call(["g++", "-std=c++14", "-O2", "-I", os.path.join(ROOT, "include"),
                           os.path.join(ROOT, "tests", "cpp", "shim_caller.cpp"), "-o", str(exe),
                           "-L", os.path.dirname(lib), "-lrangelibc_gb300", f"-Wl,-rpath,{os.path.dirname(lib)}"])
    wl = W.particle_filter_step(side=384, n_particles=500, n_beams=41, max_range_px=150.0, seed=61,
                                origin=(-2.0, -1.0))
    world = tuple(float(np.float32(v)) for v in wl.world)
    Wd, Hd = wl.occ.shape
    n, na, K = len(wl.ins), len(wl.angles), wl.table.shape[0]
    with open(tmp_path / "in.bin", "wb") as f:
        f.write(np.array([Wd, Hd], np.int32).tobytes() + wl.occ.astype(np.uint8).tobytes()
                + np.array(world, np.float32).tobytes() + np.array([n, na, K], np.int32).tobytes()
                + wl.ins.tobytes() + wl.angles.tobytes() + wl.obs.tobytes() + wl.table.tobytes())
    subprocess.check_call([str(exe), str(tmp_path / "in.bin"), str(tmp_path / "out.bin")])
    buf = open(tmp_path / "out.bin", "rb").read()
    off = 0

    def take(dtype, count):
        nonlocal off
        a = np.frombuffer(buf, dtype, count, off)
        off += a.nbytes
        return a

    bl, rm, cd, pcd = (take(np.float32, n) for _ in range(4))
    ranges = take(np.float32, n * na)
    ev, fu = take(np.float64, n), take(np.float64, n)
    dt = take(np.float32, Wd * Hd).reshape(Wd, Hd)
    raw = take(np.float32, n)
    glt = take(np.float32, n)
    lut = take(np.uint16, Wd * Hd * 36).reshape(Wd, Hd, 36)
    pair = take(np.float32, n * 2).reshape(n, 2)
    radial = take(np.float32, n * 61)
    from_json = take(np.float32, n)
    O = oracle_mod
    og = O.OracleMethod(wl.occ, "glt", 150.0, td=36, world=world, nthreads=os.cpu_count() or 1)
    assert np.array_equal(lut, og.glt_table())
    assert np.array_equal(glt, og.calc_range_many(wl.ins))
    oc = O.OracleMethod(wl.occ, "cddt", 150.0, td=108, world=world)
    exp_pair = np.array([oc.calc_range_pair(*v) for v in wl.ins], np.float32)
    assert np.array_equal(pair, exp_pair)
    exp_rad = np.full(n * 61, -7.0, np.float32)
    oc.calc_range_many_radial_optimized(61, np.float32(-2.35619449), np.float32(2.35619449), wl.ins, exp_rad)
    assert np.array_equal(radial, exp_rad)
    assert np.array_equal(dt, O.edt(wl.occ))
    for got, kind in ((bl, "bl"), (rm, "rm")):
        exp = O.OracleMethod(wl.occ, kind, 150.0, world=world).calc_range_many(wl.ins)
        assert np.mean(got != exp) < 1e-3
    for got, kind in ((cd, "cddt"), (pcd, "pcddt")):
        assert np.array_equal(got, O.OracleMethod(wl.occ, kind, 150.0, td=108, world=world).calc_range_many(wl.ins))
    # serializeJson of the pruned table: the document of the Python serialiser (pinned to the
    # reference's text at 7 digits by the CPU tests), and loadJson restores the table exactly
    op = O.OracleMethod(wl.occ, "pcddt", 150.0, td=108, world=world)
    widths, trans, bin_len, zeros = op.cddt_table()
    for suffix, prec in ((".json", 9), (".json7", 7)):
        text = open(str(tmp_path / "out.bin") + suffix).read()
        assert text == cddt_json_dumps(108, 150.0, trans, widths, bin_len, zeros, wl.occ, "", prec)
    assert np.array_equal(from_json, pcd)
    orm = O.OracleMethod(wl.occ, "rm", 150.0, world=world)
    orm.set_sensor_model(wl.table)
    assert np.mean(ranges != orm.calc_range_repeat_angles(wl.ins, wl.angles)) < 1e-3
    assert np.array_equal(ev, orm.eval_sensor_model(wl.obs, ranges, na, n))
    exp_fu = orm.calc_range_repeat_angles_eval_sensor_model(wl.ins, wl.angles, wl.obs)
    assert np.mean(np.abs(fu - exp_fu) <= 1e-6 * np.abs(exp_fu)) >= 0.99
    exp_raw = O.OracleMethod(wl.occ, "rm", 150.0).calc_range_many_raw(wl.ins)
    assert np.mean(raw != exp_raw) < 1e-3
