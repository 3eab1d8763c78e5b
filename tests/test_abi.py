"""The C-ABI library builds, loads and exports everything include/rangelibc.h declares.

No compute calls: only the checks the library makes on the host before it
touches a device (argument validation) run here.
"""
import ctypes as C
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "rangelibc.h")


def _declared():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"RLC_API\s+[\w\s\*]+?\b(rlc_\w+)\s*\(", text)))


@pytest.fixture(scope="module")
def L():
    from range_libc_gb300 import _lib
    return _lib.lib()


def test_header_declares_entry_points():
    names = _declared()
    for must in ("rlc_map_create", "rlc_method_create", "rlc_calc_range_many", "rlc_calc_range_repeat_angles",
                 "rlc_set_sensor_model", "rlc_eval_sensor_model",
                 "rlc_calc_range_repeat_angles_eval_sensor_model", "rlc_cddt_prune", "rlc_batch_run",
                 "rlc_distance_transform_noalloc", "rlc_glt_table", "rlc_cddt_calc_range_pair",
                 "rlc_cddt_calc_range_many_radial", "rlc_set_host_path", "rlc_host_path"):
        assert must in names


def test_library_exports_every_declared_symbol(L):
    from range_libc_gb300 import _lib
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.library_path()], capture_output=True, text=True)
    exported = set(re.findall(r"\bT (rlc_\w+)", out.stdout))
    missing = [n for n in _declared() if n not in exported]
    assert not missing, missing
    # and the ctypes table binds every one of them
    assert set(_declared()) <= set(_lib.SIGNATURES)


def test_abi_version(L):
    assert L.rlc_abi_version() == 1


def test_host_side_argument_checks(L):
    from range_libc_gb300 import _lib
    out = C.c_void_p()
    assert L.rlc_map_create(None, 4, 4, C.byref(out)) == _lib.RLC_ERR_ARG
    assert b"null occupancy" in L.rlc_last_error()
    occ = (C.c_uint8 * 4)()
    assert L.rlc_map_create(occ, 0, 4, C.byref(out)) == _lib.RLC_ERR_ARG
    assert L.rlc_method_create(None, 1, 10.0, 0, C.byref(out)) == _lib.RLC_ERR_ARG
    assert L.rlc_calc_range_many(None, None, None, 3, 0, None) == _lib.RLC_ERR_ARG
    assert L.rlc_batch_create(None, 0, 0, C.byref(out)) == _lib.RLC_ERR_ARG
    assert L.rlc_distance_transform_noalloc(None, 8, 8, None, None) == _lib.RLC_ERR_ARG
    assert L.rlc_map_destroy(None) == _lib.RLC_OK


def test_python_module_fails_loudly_without_a_device(L):
    import range_libc_gb300.range_libc as rl
    if rl.device_count() > 0:
        pytest.skip("a device is visible")
    with pytest.raises(rl._lib.RangeLibError):
        rl.PyOMap(4, 4)


def test_cpython_entry_points(L):
    """The CPython module of the per-call methods (csrc/rlc_py.c): it is built beside the library,
    passes the C ABI's status through (a null handle is RLC_ERR_ARG) and returns -1 -- "take the
    checked path" -- for anything that is not a C-contiguous buffer of the expected type and rank."""
    import numpy as np
    from range_libc_gb300 import _lib
    F = _lib.fast()
    assert F is not None and os.path.dirname(F.__file__) == os.path.dirname(_lib.library_path())
    ins, ang, obs = np.zeros((10, 3), np.float32), np.zeros(5, np.float32), np.zeros(5, np.float32)
    w, r = np.zeros(10, np.float64), np.zeros(50, np.float32)
    assert F.fused(0, ins, ang, obs, w) == _lib.RLC_ERR_ARG
    assert F.repeat_angles(0, ins, ang, r) == _lib.RLC_ERR_ARG
    assert F.calc_range_many(0, ins, r[:10]) == _lib.RLC_ERR_ARG
    assert F.eval_sensor_model(0, obs, r, w, 5, 10) == _lib.RLC_ERR_ARG
    assert F.fused(0, ins.astype(np.float64), ang, obs, w) == -1      # dtype
    assert F.fused(0, ins[:, :2], ang, obs, w) == -1                  # not contiguous
    assert F.fused(0, ins, ang, obs, w.astype(np.float32)) == -1      # weights must be float64
    assert F.fused(0, ins, ang, obs[:3], w) == -1                     # too few observations
    ro = np.zeros(10, np.float64)
    ro.flags.writeable = False
    assert F.fused(0, ins, ang, obs, ro) == -1                        # read-only output
    assert F.repeat_angles(0, ins, ang, [0.0] * 50) == -1             # not a buffer
