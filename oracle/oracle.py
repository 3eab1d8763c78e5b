"""ctypes front end of the CPU oracle -- TEST INFRASTRUCTURE.

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of bench.py
import this module, as the oracle that results are compared with (or as the timed CPU
baseline).  Nothing in
``range_libc_gb300`` imports it.

``Oracle*`` classes wrap ``oracle/rlc_oracle.c`` (a plain-C restatement of the
reference, kctess5/range_libc includes/RangeLib.h).  ``Ref*`` classes wrap
``oracle/_ref/librlc_ref.so``, the reference itself compiled from its sources
(only where those sources exist; the GPU host never has them).

Grid layout: ``occ[x, y]`` with shape ``(width, height)``, C order -- the
reference's ``OMap::grid[x][y]``.
"""
from __future__ import annotations

import ctypes as C
import os
import platform
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", platform.machine(), "librlc_oracle.so")
ORACLE_FAST_SO = os.path.join(HERE, "_build", platform.machine(), "librlc_oracle_fast.so")
REF_SO = os.path.join(HERE, "_ref", "librlc_ref.so")
REF_FAST_SO = os.path.join(HERE, "_ref", "librlc_ref_fast.so")


def _reference_dir() -> str:
    """Where the reference's sources lie: RLC_REFERENCE_DIR, else the oracle Makefile's REF."""
    env = os.environ.get("RLC_REFERENCE_DIR")
    if env:
        return env
    try:
        return subprocess.check_output(["make", "-s", "-C", HERE, "refdir"], text=True).strip()
    except (OSError, subprocess.CalledProcessError):
        return ""


REF_SRC = _reference_dir()

BL, RM, CDDT, GLT = 0, 1, 2, 3
KINDS = {"bl": BL, "rm": RM, "cddt": CDDT, "pcddt": CDDT, "glt": GLT}

_f32p = C.POINTER(C.c_float)
_f64p = C.POINTER(C.c_double)
_u8p = C.POINTER(C.c_uint8)
_i32p = C.POINTER(C.c_int)
_i64p = C.POINTER(C.c_int64)


def build(reference: bool | None = None) -> None:
    """Compile the oracle (always) and the reference harness (when its sources exist)."""
    subprocess.check_call(["make", "-s", "-C", HERE, "all"])
    if reference is None:
        reference = bool(REF_SRC) and os.path.isdir(os.path.join(REF_SRC, "includes"))
    if reference:
        subprocess.check_call(["make", "-s", "-C", HERE, "ref", f"REF={REF_SRC}"])


def _ptr(a: np.ndarray, t):
    return a.ctypes.data_as(t)


class _World(C.Structure):
    _fields_ = [(n, C.c_float) for n in ("scale", "angle", "origin_x", "origin_y", "sin_angle", "cos_angle")]


class _Method(C.Structure):
    _fields_ = [
        ("kind", C.c_int), ("width", C.c_int), ("height", C.c_int),
        ("occ", _u8p), ("dt", _f32p), ("cddt", C.c_void_p),
        ("max_range", C.c_float), ("world", _World),
        ("table", _f64p), ("K", C.c_int), ("glt", C.c_void_p), ("trig", _f32p),
    ]


class _Glt(C.Structure):
    _fields_ = [
        ("width", C.c_int), ("height", C.c_int), ("td", C.c_uint), ("max_range", C.c_float),
        ("td_div_2pi", C.c_float), ("twopi_div_td", C.c_float), ("max_div_limits", C.c_float),
        ("limits_div_max", C.c_float), ("lut", C.POINTER(C.c_uint16)),
    ]


class _Cddt(C.Structure):
    _fields_ = [
        ("width", C.c_int), ("height", C.c_int), ("occ", _u8p), ("max_range", C.c_float),
        ("td", C.c_uint), ("td_div_2pi", C.c_float), ("twopi_div_td", C.c_float),
        ("widths", _i32p), ("trans", _f32p), ("slice_base", _i64p), ("bin_start", _i64p),
        ("zeros", _f32p), ("total_bins", C.c_int64),
    ]


_libs = {}


def lib(fast: bool = False):
    """The strict oracle build, or (fast=True) the same code built with the reference's shipped
    flags -- a speed baseline whose results are not the oracle's."""
    key = bool(fast)
    if key not in _libs:
        path = ORACLE_FAST_SO if fast else ORACLE_SO
        if not os.path.exists(path):
            build(reference=False)
        _libs[key] = _bind(C.CDLL(path))
    return _libs[key]


def _bind(L):
    """Argument and result types of the oracle's C functions on the loaded library L."""
    L.orc_edt.argtypes = [_u8p, C.c_int, C.c_int, _f32p]
    L.orc_edge_map.argtypes = [_u8p, C.c_int, C.c_int, _u8p]
    for fn in ("orc_rm_calc_range", "orc_bl_calc_range"):
        getattr(L, fn).restype = C.c_float
    L.orc_rm_calc_range.argtypes = [_f32p, C.c_int, C.c_int, C.c_float, C.c_float, C.c_float, C.c_float, _i32p]
    L.orc_rm_calc_range_trig.argtypes = [_f32p, C.c_int, C.c_int, C.c_float, C.c_float, C.c_float, C.c_float, C.c_float, _i32p]
    L.orc_rm_calc_range_trig.restype = C.c_float
    L.orc_bl_calc_range.argtypes = [_u8p, C.c_int, C.c_int, C.c_float, C.c_float, C.c_float, C.c_float, _i32p]
    L.orc_bl_calc_range_trig.argtypes = [_u8p, C.c_int, C.c_int, C.c_float, C.c_float, C.c_float, C.c_float, C.c_float, _i32p]
    L.orc_bl_calc_range_trig.restype = C.c_float
    L.orc_cddt_build.argtypes = [_u8p, C.c_int, C.c_int, C.c_float, C.c_uint]
    L.orc_cddt_build.restype = C.POINTER(_Cddt)
    L.orc_cddt_prune.argtypes = [C.POINTER(_Cddt), C.c_float]
    L.orc_cddt_free.argtypes = [C.POINTER(_Cddt)]
    L.orc_cddt_calc_range.argtypes = [C.POINTER(_Cddt), C.c_float, C.c_float, C.c_float, _i32p]
    L.orc_cddt_calc_range.restype = C.c_float
    L.orc_cddt_num_zeros.argtypes = [C.POINTER(_Cddt)]
    L.orc_cddt_num_zeros.restype = C.c_int64
    L.orc_cddt_load.argtypes = [C.POINTER(_Cddt), _i32p, _f32p, _i64p, _f32p, C.c_int64]
    L.orc_cddt_discretize.argtypes = [C.POINTER(_Cddt), C.c_float, _i32p, _f32p, _i32p]
    mp = C.POINTER(_Method)
    L.orc_numpy_calc_range.argtypes = [mp, _f32p, _f32p, C.c_int, C.c_int]
    L.orc_calc_range_many_raw.argtypes = [mp, _f32p, _f32p, C.c_int, C.c_int]
    L.orc_numpy_calc_range_angles.argtypes = [mp, _f32p, _f32p, _f32p, C.c_int, C.c_int, C.c_int]
    L.orc_eval_sensor_model.argtypes = [mp, _f32p, _f32p, _f64p, C.c_int, C.c_int, C.c_int]
    L.orc_calc_range_repeat_angles_eval_sensor_model.argtypes = [mp, _f32p, _f32p, _f32p, _f64p, C.c_int, C.c_int, C.c_int]
    L.orc_method_calc_range.argtypes = [mp, C.c_float, C.c_float, C.c_float, _i32p]
    L.orc_method_calc_range.restype = C.c_float
    L.orc_world_rays.argtypes = [C.POINTER(_World), _f32p, _f32p, C.c_int, C.c_int, _f32p, _f32p]
    L.orc_mean_steps.argtypes = [mp, _f32p, _f32p, C.c_int, C.c_int]
    L.orc_mean_steps.restype = C.c_double
    L.orc_cddt_calc_range_pair.argtypes = [C.POINTER(_Cddt), C.c_float, C.c_float, C.c_float, _f32p, _f32p]
    L.orc_cddt_radial.argtypes = [mp, _f32p, _f32p, C.c_int, C.c_int, C.c_float, C.c_float]
    L.orc_glt_build.argtypes = [_f32p, C.c_int, C.c_int, C.c_float, C.c_uint, C.c_int]
    L.orc_glt_build.restype = C.POINTER(_Glt)
    L.orc_glt_free.argtypes = [C.POINTER(_Glt)]
    L.orc_glt_calc_range.argtypes = [C.POINTER(_Glt), C.c_float, C.c_float, C.c_float]
    L.orc_glt_calc_range.restype = C.c_float
    L.orc_glt_discretize.argtypes = [C.POINTER(_Glt), C.c_float]
    return L


def _occ(occ) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(occ) != 0, dtype=np.uint8)


def edt(occ) -> np.ndarray:
    o = _occ(occ)
    out = np.empty(o.shape, np.float32)
    if o.size:
        lib().orc_edt(_ptr(o, _u8p), o.shape[0], o.shape[1], _ptr(out, _f32p))
    return out


def edge_map(occ) -> np.ndarray:
    o = _occ(occ)
    out = np.empty(o.shape, np.uint8)
    lib().orc_edge_map(_ptr(o, _u8p), o.shape[0], o.shape[1], _ptr(out, _u8p))
    return out


def world_tuple(scale=1.0, angle=0.0, origin_x=0.0, origin_y=0.0, sin_angle=None, cos_angle=None):
    if sin_angle is None:
        sin_angle = float(np.float32(np.sin(angle)))
    if cos_angle is None:
        cos_angle = float(np.float32(np.cos(angle)))
    return (scale, angle, origin_x, origin_y, sin_angle, cos_angle)


def world_rays(world, ins, angles=None):
    """(x, y, heading) in calc_range space and (cos, sin) of every ray, as the reference forms them."""
    ins = np.ascontiguousarray(ins, np.float32)
    n = ins.shape[0]
    na = 1 if angles is None else len(angles)
    xyh = np.empty((n * na, 3), np.float32)
    trig = np.empty((n * na, 2), np.float32)
    w = _World(*world)
    ap = None
    if angles is not None:
        angles = np.ascontiguousarray(angles, np.float32)
        ap = _ptr(angles, _f32p)
    lib().orc_world_rays(C.byref(w), _ptr(ins, _f32p), ap, n, na, _ptr(xyh, _f32p), _ptr(trig, _f32p))
    return xyh, trig


class OracleMethod:
    """One of the reference's range methods, restated on the CPU.

    kind: 'bl', 'rm', 'cddt', 'pcddt' (pruned at construction) or 'glt' (GiantLUTCast with td
    angle bins, built from the distance transform with ``nthreads`` threads).  fast=True runs the
    queries on the same restatement built with the reference's shipped flags (a speed baseline:
    fast-math changes some results, so parity checks never use it).
    """

    def __init__(self, occ, kind: str, max_range: float, td: int = 108, world=None, nthreads: int = 1,
                 fast: bool = False):
        self._L = lib(fast)
        self.occ = _occ(occ)
        self.width, self.height = self.occ.shape
        self.kind_name = kind
        self.kind = KINDS[kind]
        self.max_range = float(max_range)
        self.world = world_tuple() if world is None else tuple(world)
        self.dt = edt(self.occ) if self.kind in (RM, GLT) else None
        self.glt = None
        if self.kind == GLT:
            self.glt = self._L.orc_glt_build(_ptr(self.dt, _f32p), self.width, self.height,
                                           C.c_float(self.max_range), td, nthreads)
        self.cddt = None
        if self.kind == CDDT:
            self.cddt = self._L.orc_cddt_build(_ptr(self.occ, _u8p), self.width, self.height,
                                             C.c_float(self.max_range), td)
            if kind == "pcddt":
                self.prune()
        self.table = None
        self.trig = None
        self._m = _Method()
        self._sync()

    def _sync(self):
        m = self._m
        m.kind = self.kind
        m.width, m.height = self.width, self.height
        m.occ = _ptr(self.occ, _u8p)
        m.dt = _ptr(self.dt, _f32p) if self.dt is not None else None
        m.cddt = C.cast(self.cddt, C.c_void_p) if self.cddt is not None else None
        m.max_range = self.max_range
        m.world = _World(*self.world)
        m.table = _ptr(self.table, _f64p) if self.table is not None else None
        m.K = 0 if self.table is None else self.table.shape[0]
        m.glt = C.cast(self.glt, C.c_void_p) if self.glt is not None else None
        m.trig = _ptr(self.trig, _f32p) if self.trig is not None else None

    def set_trig_override(self, trig):
        """Per-ray (cos, sin) for the batched BL/RM calls, ray-indexed like their outputs
        (None: the libm's cosf/sinf, as the reference)."""
        self.trig = None if trig is None else np.ascontiguousarray(trig, np.float32).reshape(-1, 2)
        self._sync()

    def __del__(self):
        if getattr(self, "cddt", None) is not None:
            self._L.orc_cddt_free(self.cddt)
            self.cddt = None
        if getattr(self, "glt", None) is not None:
            self._L.orc_glt_free(self.glt)
            self.glt = None

    # --- GiantLUTCast table ---
    def glt_table(self):
        """The uint16 LUT as an array [width, height, td]."""
        g = self.glt.contents
        n = g.width * g.height * g.td
        return np.ctypeslib.as_array(g.lut, (max(n, 1),))[:n].reshape(g.width, g.height, g.td).copy()

    # --- CDDT radial pairs ---
    def calc_range_pair(self, x, y, heading):
        r, ri = C.c_float(), C.c_float()
        self._L.orc_cddt_calc_range_pair(self.cddt, x, y, heading, C.byref(r), C.byref(ri))
        return r.value, ri.value

    def calc_range_many_radial_optimized(self, num_rays, min_angle, max_angle, ins, outs):
        """Fills outs [n * num_rays] in place (positions the reference does not write keep their values)."""
        ins = np.ascontiguousarray(ins, np.float32)
        assert outs.dtype == np.float32 and outs.flags.c_contiguous and outs.size == ins.shape[0] * num_rays
        self._L.orc_cddt_radial(C.byref(self._m), _ptr(ins, _f32p), _ptr(outs, _f32p), ins.shape[0], num_rays,
                              min_angle, max_angle)
        return outs

    # --- CDDT table ---
    def prune(self, max_range: float | None = None):
        self._L.orc_cddt_prune(self.cddt, C.c_float(self.max_range if max_range is None else max_range))

    def cddt_table(self):
        """(widths, trans, bin_len, zeros) of the CSR table."""
        c = self.cddt.contents
        td = c.td
        widths = np.ctypeslib.as_array(c.widths, (td,)).copy()
        trans = np.ctypeslib.as_array(c.trans, (td,)).copy()
        nb = int(c.total_bins)
        starts = np.ctypeslib.as_array(c.bin_start, (nb + 1,)).copy()
        nz = int(starts[-1])
        zeros = np.ctypeslib.as_array(c.zeros, (max(nz, 1),))[:nz].copy()
        return widths, trans, np.diff(starts), zeros

    def load_cddt_table(self, widths, trans, bin_len, zeros):
        widths = np.ascontiguousarray(widths, np.int32)
        trans = np.ascontiguousarray(trans, np.float32)
        bin_len = np.ascontiguousarray(bin_len, np.int64)
        zeros = np.ascontiguousarray(zeros, np.float32)
        rc = self._L.orc_cddt_load(self.cddt, _ptr(widths, _i32p), _ptr(trans, _f32p),
                                 _ptr(bin_len, _i64p), _ptr(zeros, _f32p), len(zeros))
        if rc != 0:
            raise ValueError(f"table shape mismatch ({rc})")

    # --- queries ---
    def calc_range(self, x, y, heading):
        return self._L.orc_method_calc_range(C.byref(self._m), x, y, heading, None)

    def calc_range_steps(self, x, y, heading):
        s = C.c_int(0)
        r = self._L.orc_method_calc_range(C.byref(self._m), x, y, heading, C.byref(s))
        return r, s.value

    def calc_range_trig(self, x, y, c, s):
        if self.kind == RM:
            return self._L.orc_rm_calc_range_trig(_ptr(self.dt, _f32p), self.width, self.height,
                                                self.max_range, x, y, c, s, None)
        if self.kind == BL:
            return self._L.orc_bl_calc_range_trig(_ptr(self.occ, _u8p), self.width, self.height,
                                                self.max_range, x, y, c, s, None)
        raise ValueError("trig parity mode applies to BL and RM")

    def calc_range_many(self, ins, nthreads=1):
        ins = np.ascontiguousarray(ins, np.float32)
        out = np.empty(ins.shape[0], np.float32)
        self._L.orc_numpy_calc_range(C.byref(self._m), _ptr(ins, _f32p), _ptr(out, _f32p), len(out), nthreads)
        return out

    def calc_range_many_raw(self, ins, nthreads=1):
        ins = np.ascontiguousarray(ins, np.float32)
        out = np.empty(ins.shape[0], np.float32)
        self._L.orc_calc_range_many_raw(C.byref(self._m), _ptr(ins, _f32p), _ptr(out, _f32p), len(out), nthreads)
        return out

    def calc_range_repeat_angles(self, ins, angles, nthreads=1):
        ins = np.ascontiguousarray(ins, np.float32)
        angles = np.ascontiguousarray(angles, np.float32)
        out = np.empty(ins.shape[0] * len(angles), np.float32)
        self._L.orc_numpy_calc_range_angles(C.byref(self._m), _ptr(ins, _f32p), _ptr(angles, _f32p),
                                          _ptr(out, _f32p), ins.shape[0], len(angles), nthreads)
        return out

    def set_sensor_model(self, table):
        self.table = np.ascontiguousarray(table, np.float64)
        self._sync()

    def eval_sensor_model(self, obs, ranges, num_rays, num_particles, nthreads=1):
        obs = np.ascontiguousarray(obs, np.float32)
        ranges = np.ascontiguousarray(ranges, np.float32)
        out = np.empty(num_particles, np.float64)
        self._L.orc_eval_sensor_model(C.byref(self._m), _ptr(obs, _f32p), _ptr(ranges, _f32p),
                                    _ptr(out, _f64p), num_rays, num_particles, nthreads)
        return out

    def calc_range_repeat_angles_eval_sensor_model(self, ins, angles, obs, nthreads=1):
        ins = np.ascontiguousarray(ins, np.float32)
        angles = np.ascontiguousarray(angles, np.float32)
        obs = np.ascontiguousarray(obs, np.float32)
        out = np.empty(ins.shape[0], np.float64)
        self._L.orc_calc_range_repeat_angles_eval_sensor_model(
            C.byref(self._m), _ptr(ins, _f32p), _ptr(angles, _f32p), _ptr(obs, _f32p),
            _ptr(out, _f64p), ins.shape[0], len(angles), nthreads)
        return out

    def mean_steps(self, ins, angles=None):
        ins = np.ascontiguousarray(ins, np.float32)
        ap = None
        if angles is not None:
            angles = np.ascontiguousarray(angles, np.float32)
            ap = _ptr(angles, _f32p)
        return self._L.orc_mean_steps(C.byref(self._m), _ptr(ins, _f32p), ap, ins.shape[0],
                                    1 if angles is None else len(angles))


# ---------------------------------------------------------------------------
# The reference itself (compiled from its sources; dev container only)
# ---------------------------------------------------------------------------
_ref = {}


def ref_available(fast: bool = False) -> bool:
    return os.path.exists(REF_FAST_SO if fast else REF_SO)


def ref_lib(fast: bool = False):
    key = bool(fast)
    if key not in _ref:
        L = C.CDLL(REF_FAST_SO if fast else REF_SO)
        vp = C.c_void_p
        L.ref_map_create.argtypes = [_u8p, C.c_int, C.c_int] + [C.c_float] * 6
        L.ref_map_create.restype = vp
        L.ref_map_destroy.argtypes = [vp]
        L.ref_map_load_png.argtypes = [C.c_char_p, C.c_float, _i32p, _i32p]
        L.ref_map_load_png.restype = vp
        L.ref_map_grid.argtypes = [vp, _u8p]
        L.ref_dt.argtypes = [vp, _f32p]
        L.ref_edge_map.argtypes = [vp, _u8p]
        L.ref_method_create.argtypes = [vp, C.c_int, C.c_float, C.c_uint]
        L.ref_method_create.restype = vp
        L.ref_method_destroy.argtypes = [vp]
        L.ref_calc_range.argtypes = [vp, C.c_float, C.c_float, C.c_float]
        L.ref_calc_range.restype = C.c_float
        L.ref_calc_range_many_raw.argtypes = [vp, _f32p, _f32p, C.c_int]
        L.ref_numpy_calc_range.argtypes = [vp, _f32p, _f32p, C.c_int]
        L.ref_numpy_calc_range_angles.argtypes = [vp, _f32p, _f32p, _f32p, C.c_int, C.c_int]
        L.ref_set_sensor_model.argtypes = [vp, _f64p, C.c_int]
        L.ref_eval_sensor_model.argtypes = [vp, _f32p, _f32p, _f64p, C.c_int, C.c_int]
        L.ref_fused.argtypes = [vp, _f32p, _f32p, _f32p, _f64p, C.c_int, C.c_int]
        L.ref_cddt_prune.argtypes = [vp, C.c_float]
        L.ref_cddt_num_zeros.argtypes = [vp]
        L.ref_cddt_num_zeros.restype = C.c_longlong
        L.ref_cddt_num_bins.argtypes = [vp]
        L.ref_cddt_num_bins.restype = C.c_longlong
        L.ref_cddt_export.argtypes = [vp, _i32p, _f32p, _i64p, _f32p]
        L.ref_cddt_pair.argtypes = [vp, C.c_float, C.c_float, C.c_float, _f32p, _f32p]
        L.ref_cddt_radial.argtypes = [vp, _f32p, _f32p, C.c_int, C.c_int, C.c_float, C.c_float]
        L.ref_glt_slice.argtypes = [vp, C.c_float, _f32p]
        L.ref_cddt_json.argtypes = [vp, C.c_char_p, C.c_longlong]
        L.ref_cddt_json.restype = C.c_longlong
        _ref[key] = L
    return _ref[key]


class RefMap:
    def __init__(self, occ=None, world=None, png=None, threshold=128.0, fast=False):
        self.L = ref_lib(fast)
        if png is not None:
            w, h = C.c_int(0), C.c_int(0)
            self.h = self.L.ref_map_load_png(png.encode(), threshold, C.byref(w), C.byref(h))
            if not self.h:
                raise IOError(png)
            self.occ = np.empty((w.value, h.value), np.uint8)
            self.L.ref_map_grid(self.h, _ptr(self.occ, _u8p))
            self.world = world_tuple()
        else:
            self.occ = _occ(occ)
            self.world = world_tuple() if world is None else tuple(world)
            self.h = self.L.ref_map_create(_ptr(self.occ, _u8p), self.occ.shape[0], self.occ.shape[1], *self.world)

    def __del__(self):
        if getattr(self, "h", None):
            self.L.ref_map_destroy(self.h)
            self.h = None

    def dt(self):
        out = np.empty(self.occ.shape, np.float32)
        self.L.ref_dt(self.h, _ptr(out, _f32p))
        return out

    def edge_map(self):
        out = np.empty(self.occ.shape, np.uint8)
        self.L.ref_edge_map(self.h, _ptr(out, _u8p))
        return out


class RefMethod:
    def __init__(self, rmap: RefMap, kind: str, max_range: float, td: int = 108):
        self.map = rmap
        self.L = rmap.L
        self.kind = KINDS[kind]
        self.max_range = float(max_range)
        self.td = int(td)
        self.h = self.L.ref_method_create(rmap.h, self.kind, self.max_range, td)
        if kind == "pcddt":
            self.prune()

    def __del__(self):
        if getattr(self, "h", None):
            self.L.ref_method_destroy(self.h)
            self.h = None

    def prune(self, max_range=None):
        self.L.ref_cddt_prune(self.h, self.max_range if max_range is None else max_range)

    def calc_range(self, x, y, h):
        return self.L.ref_calc_range(self.h, x, y, h)

    def calc_range_pair(self, x, y, heading):
        r, ri = C.c_float(), C.c_float()
        self.L.ref_cddt_pair(self.h, x, y, heading, C.byref(r), C.byref(ri))
        return r.value, ri.value

    def calc_range_many_radial_optimized(self, num_rays, min_angle, max_angle, ins, outs):
        ins = np.ascontiguousarray(ins, np.float32)
        self.L.ref_cddt_radial(self.h, _ptr(ins, _f32p), _ptr(outs, _f32p), ins.shape[0], num_rays,
                               min_angle, max_angle)
        return outs

    def glt_table(self):
        """The LUT as [width, height, td] (the reference's get_slice per angle bin)."""
        w, h = self.map.occ.shape
        out = np.empty((self.td, w, h), np.float32)
        for i in range(self.td):
            theta = float(np.float32(i) * np.float32(6.28318530718 / np.float32(self.td)))
            self.L.ref_glt_slice(self.h, theta, _ptr(out[i], _f32p))
        return np.moveaxis(out, 0, 2).astype(np.uint16)

    def calc_range_many(self, ins):
        ins = np.ascontiguousarray(ins, np.float32)
        out = np.empty(ins.shape[0], np.float32)
        self.L.ref_numpy_calc_range(self.h, _ptr(ins, _f32p), _ptr(out, _f32p), len(out))
        return out

    def calc_range_many_raw(self, ins):
        ins = np.ascontiguousarray(ins, np.float32)
        out = np.empty(ins.shape[0], np.float32)
        self.L.ref_calc_range_many_raw(self.h, _ptr(ins, _f32p), _ptr(out, _f32p), len(out))
        return out

    def calc_range_repeat_angles(self, ins, angles):
        ins = np.ascontiguousarray(ins, np.float32)
        angles = np.ascontiguousarray(angles, np.float32)
        out = np.empty(ins.shape[0] * len(angles), np.float32)
        self.L.ref_numpy_calc_range_angles(self.h, _ptr(ins, _f32p), _ptr(angles, _f32p), _ptr(out, _f32p),
                                           ins.shape[0], len(angles))
        return out

    def set_sensor_model(self, table):
        self.table = np.ascontiguousarray(table, np.float64)
        self.L.ref_set_sensor_model(self.h, _ptr(self.table, _f64p), self.table.shape[0])

    def eval_sensor_model(self, obs, ranges, num_rays, num_particles):
        obs = np.ascontiguousarray(obs, np.float32)
        ranges = np.ascontiguousarray(ranges, np.float32)
        out = np.empty(num_particles, np.float64)
        self.L.ref_eval_sensor_model(self.h, _ptr(obs, _f32p), _ptr(ranges, _f32p), _ptr(out, _f64p),
                                     num_rays, num_particles)
        return out

    def calc_range_repeat_angles_eval_sensor_model(self, ins, angles, obs):
        ins = np.ascontiguousarray(ins, np.float32)
        angles = np.ascontiguousarray(angles, np.float32)
        obs = np.ascontiguousarray(obs, np.float32)
        out = np.empty(ins.shape[0], np.float64)
        self.L.ref_fused(self.h, _ptr(ins, _f32p), _ptr(angles, _f32p), _ptr(obs, _f32p), _ptr(out, _f64p),
                         ins.shape[0], len(angles))
        return out

    def cddt_table(self):
        nb = int(self.L.ref_cddt_num_bins(self.h))
        nz = int(self.L.ref_cddt_num_zeros(self.h))
        widths = np.zeros(self.td, np.int32)
        trans = np.zeros(self.td, np.float32)
        bin_len = np.zeros(max(nb, 1), np.int64)
        zeros = np.zeros(max(nz, 1), np.float32)
        self.L.ref_cddt_export(self.h, _ptr(widths, _i32p), _ptr(trans, _f32p), _ptr(bin_len, _i64p),
                               _ptr(zeros, _f32p))
        return widths, trans, bin_len[:nb].copy(), zeros[:nz].copy()

    def cddt_json(self) -> str:
        """The reference's CDDTCast::serializeJson document."""
        n = int(self.L.ref_cddt_json(self.h, None, 0))
        buf = C.create_string_buffer(n)
        self.L.ref_cddt_json(self.h, buf, n)
        return buf.raw[:n].decode()
