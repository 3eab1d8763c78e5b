"""Loader of the CUDA library (``_build/librangelibc_gb300.so``) and its C ABI.

The library is the only compute path: there is no CPU fallback.  If the
shared object is missing it is built with nvcc (``build.py``); if that is not
possible, or the ABI does not match, loading raises.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

from .build import LIB_PATH as _LIB_PATH, build as _build_library, fast_module_path as _fast_module_path

RLC_OK, RLC_ERR_ARG, RLC_ERR_CUDA, RLC_ERR_STATE, RLC_ERR_NOMEM, RLC_ERR_IO = range(6)
RLC_BL, RLC_RM, RLC_CDDT, RLC_PCDDT, RLC_RMGPU, RLC_GLT = range(6)
RLC_DEVICE_PTRS = 1
RLC_HOST_AUTO, RLC_HOST_STAGED = 0, 1
RLC_NO_WORLD = 2
RLC_TUNE_FLUSH_L2 = 1
ABI_VERSION = 1

_f32p = C.POINTER(C.c_float)
_f64p = C.POINTER(C.c_double)
_u8p = C.POINTER(C.c_uint8)
_i32p = C.POINTER(C.c_int)
_i64p = C.POINTER(C.c_int64)
_u32p = C.POINTER(C.c_uint)
_vp = C.c_void_p


class RangeLibError(RuntimeError):
    """A C-ABI call returned an error status."""

    def __init__(self, code: int, message: str):
        super().__init__(f"[rlc status {code}] {message}")
        self.code = code


class FilterDesc(C.Structure):
    _fields_ = [
        ("method", _vp), ("ins", _vp), ("angles", _vp), ("obs", _vp),
        ("ranges", _vp), ("weights", _vp), ("n_particles", C.c_int), ("n_angles", C.c_int),
    ]


# name -> (restype, argtypes); every function returns an int status unless noted
SIGNATURES = {
    "rlc_abi_version": (C.c_int, []),
    "rlc_last_error": (C.c_char_p, []),
    "rlc_device_count": (C.c_int, []),
    "rlc_map_create": (C.c_int, [_u8p, C.c_int, C.c_int, C.POINTER(_vp)]),
    "rlc_png_occupancy": (C.c_int, [C.c_char_p, C.c_float, _vp, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "rlc_png_save_occupancy": (C.c_int, [C.c_char_p, _vp, C.c_int, C.c_int]),
    "rlc_map_set_world": (C.c_int, [_vp] + [C.c_float] * 6),
    "rlc_map_destroy": (C.c_int, [_vp]),
    "rlc_map_size": (C.c_int, [_vp, _i32p, _i32p]),
    "rlc_map_occupancy": (C.c_int, [_vp, _u8p]),
    "rlc_map_distance_transform": (C.c_int, [_vp, _f32p]),
    "rlc_map_edge_map": (C.c_int, [_vp, _u8p]),
    "rlc_method_create": (C.c_int, [_vp, C.c_int, C.c_float, C.c_uint, C.POINTER(_vp)]),
    "rlc_method_create_cddt_trig": (C.c_int, [_vp, C.c_int, C.c_float, C.c_uint, _f32p, _f32p, C.POINTER(_vp)]),
    "rlc_method_destroy": (C.c_int, [_vp]),
    "rlc_method_info": (C.c_int, [_vp, _i32p, _f32p, _u32p]),
    "rlc_method_device_flags": (C.c_int, [_vp, _u32p]),
    "rlc_cddt_prune": (C.c_int, [_vp, C.c_float]),
    "rlc_cddt_table_size": (C.c_int, [_vp, _i64p, _i64p]),
    "rlc_cddt_table_export": (C.c_int, [_vp, _i32p, _f32p, _i64p, _f32p]),
    "rlc_cddt_table_load": (C.c_int, [_vp, _f32p, _i64p, _f32p, C.c_int64]),
    "rlc_glt_table": (C.c_int, [_vp, C.POINTER(C.c_uint16)]),
    "rlc_set_host_path": (C.c_int, [C.c_int]),
    "rlc_host_path": (C.c_int, [_i32p]),
    "rlc_cddt_calc_range_pair": (C.c_int, [_vp, C.c_float, C.c_float, C.c_float, _f32p, _f32p]),
    "rlc_cddt_calc_range_many_radial": (C.c_int, [_vp, _vp, _vp, C.c_int, C.c_int, C.c_float, C.c_float,
                                                  C.c_uint, _vp]),
    "rlc_calc_range": (C.c_int, [_vp, C.c_float, C.c_float, C.c_float, _f32p]),
    "rlc_calc_range_many": (C.c_int, [_vp, _vp, _vp, C.c_int, C.c_uint, _vp]),
    "rlc_calc_range_repeat_angles": (C.c_int, [_vp, _vp, _vp, _vp, C.c_int, C.c_int, C.c_uint, _vp]),
    "rlc_set_sensor_model": (C.c_int, [_vp, _f64p, C.c_int]),
    "rlc_eval_sensor_model": (C.c_int, [_vp, _vp, _vp, _vp, C.c_int, C.c_int, C.c_uint, _vp]),
    "rlc_calc_range_repeat_angles_eval_sensor_model": (
        C.c_int, [_vp, _vp, _vp, _vp, _vp, C.c_int, C.c_int, C.c_uint, _vp]),
    "rlc_method_set_trig_override": (C.c_int, [_vp, _f32p, C.c_int64]),
    "rlc_count_steps": (C.c_int, [_vp, _vp, _vp, C.c_int, C.c_int, C.c_uint, _i64p]),
    "rlc_trig_eval": (C.c_int, [_vp, _vp, C.c_int64, C.c_uint, _vp]),
    "rlc_method_set_schedule": (C.c_int, [_vp, C.c_int, C.c_int, C.c_int, C.c_int]),
    "rlc_method_get_schedule": (C.c_int, [_vp, _i32p, _i32p, _i32p, _i32p]),
    "rlc_method_autotune": (C.c_int, [_vp, _vp, _vp, _vp, _vp, C.c_int, C.c_int, _vp]),
    "rlc_method_autotune_ex": (C.c_int, [_vp, _vp, _vp, _vp, _vp, C.c_int, C.c_int, C.c_uint, _vp]),
    "rlc_method_autotune_results": (C.c_int, [_vp, C.c_int, _i32p, _vp, _vp]),
    "rlc_distance_transform_noalloc": (C.c_int, [_vp, C.c_int, C.c_int, _vp, _vp]),
    "rlc_learned_create": (C.c_int, [_vp, C.c_uint, C.POINTER(_vp)]),
    "rlc_learned_destroy": (C.c_int, [_vp]),
    "rlc_learned_param_count": (C.c_int64, []),
    "rlc_learned_get_params": (C.c_int, [_vp, _f32p]),
    "rlc_learned_set_params": (C.c_int, [_vp, _f32p]),
    "rlc_learned_sample_rays": (C.c_int, [_vp, C.c_longlong, C.c_uint, C.c_int, _vp, _vp, _vp, _vp]),
    "rlc_learned_train": (C.c_int, [_vp, C.c_int, C.c_int, C.c_float, C.c_uint, _f32p, _vp]),
    "rlc_learned_predict": (C.c_int, [_vp, _vp, C.c_int, _vp, _vp]),
    "rlc_learned_predict_layered": (C.c_int, [_vp, _vp, C.c_int, _vp, _vp]),
    "rlc_learned_calc_range_repeat_angles": (C.c_int, [_vp, _vp, _vp, _vp, C.c_int, C.c_int, _vp, _i64p, _vp]),
    "rlc_learned_features": (C.c_int, [_vp, _vp, C.c_int, _vp]),
    "rlc_learned_gradients": (C.c_int, [_vp, _vp, _vp, C.c_int, _f32p, _f32p]),
    "rlc_tc_gemm": (C.c_int, [_vp, _vp, _vp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _vp]),
    "rlc_batch_create": (C.c_int, [C.POINTER(FilterDesc), C.c_int, C.c_int, C.POINTER(_vp)]),
    "rlc_batch_run": (C.c_int, [_vp, _vp]),
    "rlc_batch_set_schedule": (C.c_int, [_vp, C.c_int, C.c_int, C.c_int, C.c_int]),
    "rlc_batch_set_product_mode": (C.c_int, [_vp, C.c_int]),
    "rlc_batch_get_product_mode": (C.c_int, [_vp, _i32p]),
    "rlc_batch_get_schedule": (C.c_int, [_vp, _i32p, _i32p, _i32p, _i32p]),
    "rlc_batch_autotune": (C.c_int, [_vp, _vp]),
    "rlc_batch_destroy": (C.c_int, [_vp]),
    "rlc_batch_info": (C.c_int, [_vp, _i64p, _i64p]),
}

_lock = threading.Lock()
_lib = None


def library_path() -> str:
    return _LIB_PATH


def lib():
    """The loaded C ABI (built on first use if the toolkit is present)."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            path = _LIB_PATH
            if not os.path.exists(path):
                _build_library()
            L = C.CDLL(path)
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            v = L.rlc_abi_version()
            if v != ABI_VERSION:
                raise RuntimeError(f"{path}: ABI version {v}, expected {ABI_VERSION}")
            _lib = L
    return _lib


_fast = None   # None: not looked for yet; False: not built


def fast():
    """The CPython entry points of the per-call methods (csrc/rlc_py.c), or None where they were
    not built.  They call the same C ABI; -1 from them means "argument not a plain buffer of the
    expected type and shape", and the caller takes its checked ctypes path."""
    global _fast
    if _fast is None:
        lib()   # the library first, so that the module binds to this loaded copy
        mod = False
        path = _fast_module_path()
        if os.path.exists(path):
            import importlib.util
            try:
                spec = importlib.util.spec_from_file_location("_rlcfast", path)
                m = importlib.util.module_from_spec(spec)
                spec.loader.exec_module(m)
                mod = m
            except ImportError:
                mod = False
        _fast = mod
    return _fast or None


def check(rc: int) -> None:
    if rc != RLC_OK:
        msg = lib().rlc_last_error()
        raise RangeLibError(rc, msg.decode() if msg else "")


def call(name: str, *args) -> None:
    check(getattr(lib(), name)(*args))
