"""The per-ray cos/sin of the production BL and RM casts (range_libc_gb300/csrc/rlc_trig.cuh).

The reference takes each ray's cosf/sinf from the host C library (RangeLib.h:700-702, 930-931).
Without a trig override the casts here use the correctly rounded values (the floats nearest to
the exact sine and cosine).  The CPU tests build the same header for the host and compare it
with the long-double libm rounded to float; the GPU test compares the device's values with the
host build's, bit for bit.  The oracle's per-ray override (used by the production parity
tests) is checked to equal its libm path when fed the libm's own values.
"""
import os
import subprocess

import numpy as np
import pytest

from range_libc_gb300 import workloads as W

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def trig_check(tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("trig") / "trig_check")
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-o", exe,
                           os.path.join(ROOT, "tests", "cpp", "trig_check.cpp"), "-lpthread"])
    return exe


def _scan(exe, lo, hi, stride):
    import json
    out = subprocess.run([exe, "scan", str(lo), str(hi), str(stride), str(os.cpu_count() or 1)],
                         capture_output=True, text=True)
    res = json.loads(out.stdout)
    assert out.returncode == 0 and res["mismatch"] == 0, (out.stdout, out.stderr[-2000:])
    return res


def test_host_build_is_correctly_rounded(trig_check):
    """Every 127th float of [-16, 16] and every 4099th of [-4096, 4096] (the fast path), and a
    sample beyond (the double fallback).  A one-off run over all 2,197,815,296 floats of
    [-16, 16] found no mismatch (15,832 fallbacks; glibc's sinf/cosf not nearest on
    2,356,992 / 1,195,132 of them)."""
    r = _scan(trig_check, -16, 16, 127)
    assert r["n"] > 17_000_000 and r["fallback"] < r["n"] * 1e-4
    _scan(trig_check, -4096, 4096, 4099)
    _scan(trig_check, 4096, 1e7, 100003)
    _scan(trig_check, -1e7, -4096, 100003)


def test_difference_formula_is_correctly_rounded(trig_check):
    """The batch's per-ray cos/sin from float pairs of the particle heading's and the beam angle's
    sin and cos (rlc_trig::sincos_diff, with its rounding check) against the correctly rounded
    values of fl(th - a), bit for bit, on 32 M random pairs: workload-like headings and beams, wide
    arguments, differences near multiples of pi / 2 and beams that nearly cancel the heading (the
    check then declines and the caller computes the values directly)."""
    import json
    nt = max(1, min(16, os.cpu_count() or 1))
    out = subprocess.run([trig_check, "diff", str(8_000_000 // nt), str(nt)], capture_output=True, text=True)
    res = json.loads(out.stdout)
    assert out.returncode == 0 and res["mismatch"] == 0, (out.stdout, out.stderr[-2000:])
    assert res["n"] >= 30_000_000 and res["fallback"] + res["no_pair"] < res["n"] // 2


def _host_eval(exe, x):
    x = np.ascontiguousarray(x, np.float32)
    out = subprocess.run([exe, "eval"], input=x.tobytes(), capture_output=True, check=True)
    return np.frombuffer(out.stdout, np.float32).reshape(-1, 2)


def _sample():
    rng = np.random.default_rng(17)
    bits = np.arange(int(np.float32(16).view(np.uint32)), 0, -509, dtype=np.int64)
    xs = [np.concatenate([bits, bits | 0x80000000]).astype(np.uint32).view(np.float32),
          rng.uniform(-4096, 4096, 500_000).astype(np.float32),
          rng.uniform(-11.0, 0.0, 500_000).astype(np.float32),
          np.array([0.0, -0.0, 2.0 ** -12, -(2.0 ** -12), 2.0 ** -13, 1e-30, 4096.0, -4096.0, 4095.9998,
                    1e6, -3e7, 1e30, np.pi / 2, np.pi, 3 * np.pi / 2], np.float32)]
    return np.concatenate(xs)


def test_oracle_override_with_libm_values_changes_nothing(oracle_mod):
    wl = W.particle_filter_step(side=256, n_particles=50, n_beams=19, max_range_px=80.0, seed=9)
    for kind in ("rm", "bl"):
        ref = oracle_mod.OracleMethod(wl.occ, kind, wl.max_range, world=wl.world)
        ref.set_sensor_model(wl.table)
        r0 = ref.calc_range_repeat_angles(wl.ins, wl.angles)
        w0 = ref.calc_range_repeat_angles_eval_sensor_model(wl.ins, wl.angles, wl.obs)
        _, trig = oracle_mod.world_rays(wl.world, wl.ins, wl.angles)
        ref.set_trig_override(trig)
        assert np.array_equal(ref.calc_range_repeat_angles(wl.ins, wl.angles).view(np.uint32), r0.view(np.uint32))
        assert np.array_equal(ref.calc_range_repeat_angles_eval_sensor_model(wl.ins, wl.angles, wl.obs), w0)
        # a different override changes some ranges: the override is used
        ref.set_trig_override(np.roll(trig, 1, axis=0))
        assert not np.array_equal(ref.calc_range_repeat_angles(wl.ins, wl.angles), r0)


@pytest.mark.gpu
def test_device_trig_equals_host_build(rl, trig_check):
    """The device's per-ray cos/sin (rlc_trig_eval) equal the host build of the same code on
    ~5.3 M arguments: a strided walk over [-16, 16], uniform samples over the fast path's range
    and the headings of the particle-filter workloads, and edge cases (fallback included)."""
    x = _sample()
    dev = np.empty((len(x), 2), np.float32)
    rl._lib.call("rlc_trig_eval", x.ctypes.data, dev.ctypes.data, len(x), 0, None)
    host = _host_eval(trig_check, x)
    assert host.shape == dev.shape
    same = dev.view(np.uint32) == host.view(np.uint32)
    finite = np.isfinite(x)
    assert same[finite].all(), f"{int((~same[finite]).sum())} of {int(finite.sum())} values differ"
    # sin is sin, cos is cos (order of the pair), against numpy's double sine rounded
    probe = np.abs(x) < 64
    s64 = np.sin(x[probe].astype(np.float64)).astype(np.float32)
    assert np.mean(dev[probe, 0] == s64) > 0.999999
