"""Python face of the GB300 library, mirroring range_libc's Cython module.

Class and method names, argument order and meaning follow the reference's
``pywrapper/RangeLibc.pyx`` (kctess5/range_libc) so that existing callers
(particle filters written against ``range_libc``) switch by changing the
import::

    import range_libc_gb300.range_libc as range_libc
    m = range_libc.PyOMap(occupancy_bool_array)
    rm = range_libc.PyRayMarchingGPU(m, 200)
    rm.set_sensor_model(table)
    rm.calc_range_repeat_angles_eval_sensor_model(particles, angles, obs, weights)

Every call runs on the GPU through the C ABI (include/rangelibc.h).
Arrays may be numpy arrays (host memory; the call is synchronous, like the
reference) or CUDA torch tensors (device memory; the call is queued on the
current torch stream and returns immediately).  Dtypes and layouts are
those of the reference's typed buffers: float32 C-contiguous poses
``[N, 3]``, float32 angles/observations/ranges, float64 weights and tables.
"""
from __future__ import annotations

import ctypes as C
import sys

import numpy as np

from . import _lib
from ._lib import call, lib

# module flags of the reference (RangeLibc.pyx:94-102), for the shipped build
USE_CACHED_TRIG = False
USE_ALTERNATE_MOD = True
USE_CACHED_CONSTANTS = True
USE_FAST_ROUND = False
NO_INLINE = False
USE_LRU_CACHE = False
LRU_CACHE_SIZE = 1000000
SHOULD_USE_CUDA = True


# ---------------------------------------------------------------- arrays
def _is_device(a) -> bool:
    return getattr(a, "is_cuda", False) is True


def _stream_of(a):
    import torch  # device arrays are torch tensors
    return C.c_void_p(torch.cuda.current_stream(a.device).cuda_stream)


_TORCH_DTYPES = {np.float32: "torch.float32", np.float64: "torch.float64"}
_NP_DTYPES = {np.float32: np.dtype(np.float32), np.float64: np.dtype(np.float64)}


def _arg(a, dtype, ndim: int, name: str):
    """(address, is_device) of a reference-typed buffer; raises like a Cython typed buffer."""
    if isinstance(a, np.ndarray):
        if a.dtype is not _NP_DTYPES[dtype] and a.dtype != dtype:
            raise ValueError(f"Buffer dtype mismatch for {name}: expected {np.dtype(dtype).name}, got {a.dtype.name}")
        if a.ndim != ndim:
            raise ValueError(f"Buffer has wrong number of dimensions for {name} (expected {ndim}, got {a.ndim})")
        if not a.flags.c_contiguous:
            raise ValueError(f"{name} must be C-contiguous")
        try:   # the buffer protocol is ~2x quicker than ndarray.ctypes
            return C.addressof(C.c_char.from_buffer(a)), False
        except (TypeError, ValueError):   # read-only or empty arrays
            return a.ctypes.data, False
    if _is_device(a):
        if str(a.dtype) != _TORCH_DTYPES[dtype]:
            raise ValueError(f"Buffer dtype mismatch for {name}: expected {np.dtype(dtype).name}, got {a.dtype}")
        if a.dim() != ndim:
            raise ValueError(f"Buffer has wrong number of dimensions for {name} (expected {ndim}, got {a.dim()})")
        if not a.is_contiguous():
            raise ValueError(f"{name} must be C-contiguous")
        return a.data_ptr(), True
    raise TypeError(f"{name} must be a numpy.ndarray or a CUDA tensor")


def _flags_stream(dev_flags, first):
    if True not in dev_flags:
        return 0, None
    if False in dev_flags:
        raise ValueError("all arrays of one call must be host (numpy) or all device (CUDA) arrays")
    return _lib.RLC_DEVICE_PTRS, _stream_of(first)


# ---------------------------------------------------------------- PNG
def png_occupancy(path: str, threshold: float = 128.0) -> np.ndarray:
    """grid[x][y] of OMap(path, threshold) (RangeLib.h:158-201) as uint8 (width, height).

    Decoded by the library (host code, rlc_png_occupancy): pixel (x, y) is occupied when
    (int)rgb2gray(r, g, b) < threshold with r, g, b its blue, green and red bytes, as the
    reference reads them.  Raises RangeLibError for files that cannot be read or decoded.
    """
    w, h = C.c_int(0), C.c_int(0)
    p = path.encode() if isinstance(path, str) else bytes(path)
    call("rlc_png_occupancy", p, float(threshold), None, C.byref(w), C.byref(h))
    occ = np.empty((w.value, h.value), np.uint8)
    call("rlc_png_occupancy", p, float(threshold), occ.ctypes.data, C.byref(w), C.byref(h))
    return occ


# ---------------------------------------------------------------- CDDT table JSON
def _fmt_floats(vals, precision: int) -> str:
    f = "%%.%dg" % precision
    return "[" + ",".join(f % v for v in np.asarray(vals, np.float32).astype(np.float64).tolist()) + "]"


def cddt_json_dumps(theta_disc: int, max_range: float, trans, widths, bin_len, zeros, occ, path: str = "",
                    precision: int = 9) -> str:
    """A CDDT table as the document CDDTCast::serializeJson writes (RangeLib.h:1690-1735).

    Same keys, nesting, line breaks and indentation; ``map.data[x]`` is grid[x] (one 0/1 per y),
    ``compressed_lut[a]`` holds slice a's ``theta`` (a * float(2pi / td), in float like the
    reference) and its bins' zero points.  The reference prints 7 significant digits, which does
    not restore every float32; the default here is 9, which does (``cddt_json_loads`` gives the
    table back bit for bit).  With ``precision=7`` the text is the reference's, byte for byte --
    including the comma after the map's ``data`` array, which strict JSON parsers reject and
    ``cddt_json_loads`` accepts.
    """
    td = int(theta_disc)
    widths = np.asarray(widths, np.int64)
    bin_len = np.asarray(bin_len, np.int64)
    zeros = np.asarray(zeros, np.float32)
    occ = np.asarray(occ)
    if widths.shape != (td,) or int(widths.sum()) != len(bin_len) or int(bin_len.sum()) != len(zeros):
        raise ValueError("table arrays do not describe theta_disc slices")
    f = "%%.%dg" % precision
    W, H = occ.shape
    rows = np.full((W, max(2 * H - 1, 0)), ord(","), np.uint8)
    rows[:, 0::2] = (occ != 0).astype(np.uint8) + ord("0")
    data = ",".join("[" + r.tobytes().decode() + "]" if H else "[]" for r in rows)
    step = np.float32(6.28318530718 / float(np.float32(td)))
    out = ['{"cddt": {\n',
           '  "theta_discretization": %d,\n' % td,
           '  "lut_translations": %s,\n' % _fmt_floats(trans, precision),
           '  "max_range":%s,\n' % (f % float(np.float32(max_range))),
           '  "map": {\n',
           '    "path": "%s",\n' % path,
           '    "width": %d,\n' % W,
           '    "height": %d,\n' % H,
           '    "data": [%s],\n' % data,
           '  },\n',
           '  "compressed_lut": [\n']
    b = z = 0
    for a in range(td):
        theta = float(np.float32(a) * step)
        bins = []
        for _ in range(int(widths[a])):
            n = int(bin_len[b])
            bins.append(_fmt_floats(zeros[z:z + n], precision))
            b += 1
            z += n
        out.append('    {\n      "theta": %s,\n      "zeros": [%s]\n    }%s\n'
                   % (f % theta, ",".join(bins), "" if a == td - 1 else ","))
    out.append("  ]\n}}\n")
    return "".join(out)


def cddt_json_loads(text: str) -> dict:
    """Parse a document written by ``cddt_json_dumps`` or the reference's serializeJson into
    ``theta_disc, max_range, trans, widths, bin_len, zeros`` (the CSR table), ``occ`` (grid[x][y],
    uint8) and ``path``."""
    import json
    import re
    doc = json.loads(re.sub(r",(\s*[}\]])", r"\1", text))["cddt"]
    td = int(doc["theta_discretization"])
    lut = doc["compressed_lut"]
    if len(lut) != td or len(doc["lut_translations"]) != td:
        raise ValueError("compressed_lut / lut_translations do not hold theta_discretization slices")
    widths = np.array([len(s["zeros"]) for s in lut], np.int32)
    bins = [b for s in lut for b in s["zeros"]]
    bin_len = np.array([len(b) for b in bins], np.int64)
    zeros = np.array([v for b in bins for v in b], np.float64).astype(np.float32)
    m = doc["map"]
    W, H = int(m["width"]), int(m["height"])
    occ = np.array(m["data"], np.uint8).reshape(W, H) if W and H else np.zeros((W, H), np.uint8)
    return {"theta_disc": td, "max_range": float(np.float32(doc["max_range"])),
            "trans": np.array(doc["lut_translations"], np.float64).astype(np.float32),
            "widths": widths, "bin_len": bin_len, "zeros": zeros, "occ": occ, "path": m.get("path", "")}


def _quaternion_yaw(q) -> float:
    """Yaw of a geometry_msgs/Quaternion-shaped object, as the reference's quaternion_to_angle
    (RangeLibc.pyx:122-128) gets it from ROS tf.transformations.euler_from_quaternion with its
    default axes 'sxyz': the quaternion (x, y, z, w) is scaled by sqrt(2 / |q|^2), the rotation
    matrix's entries M[0][0] = 1 - q_y^2 - q_z^2 and M[1][0] = q_x q_y + q_z q_w are formed from
    the scaled components, and the yaw is atan2(M[1][0], M[0][0]) -- 0 for a near-zero quaternion
    (identity matrix) and at gimbal lock (sqrt(M[0][0]^2 + M[1][0]^2) <= 4 eps)."""
    eps = float(np.finfo(np.float64).eps) * 4.0
    v = np.array([q.x, q.y, q.z, q.w], np.float64)
    n = float(np.dot(v, v))
    if n < eps:
        return 0.0
    v *= np.sqrt(2.0 / n)
    m00 = 1.0 - v[1] * v[1] - v[2] * v[2]
    m10 = v[0] * v[1] + v[2] * v[3]
    if not np.sqrt(m00 * m00 + m10 * m10) > eps:
        return 0.0
    return float(np.arctan2(m10, m00))


def occupancy_grid_parts(msg):
    """Grid and world parameters of a nav_msgs/OccupancyGrid-shaped message, as PyOMap's ROS
    branch builds them (RangeLibc.pyx:146-167): ``data`` reshaped to (height, width) rows, a cell
    occupied when its value is > 10 (-1 unknown and 0..10 free), OMap(height, width) so that
    grid[x][y] = data[x, y] (x the row); world scale = resolution, angle = -yaw of the origin's
    orientation, origin = the origin's position, and the angle's sine and cosine.  Returns
    (occ[x, y] uint8 of shape (height, width), world tuple)."""
    info = msg.info
    width, height = int(info.width), int(info.height)
    arr = np.asarray(msg.data, dtype=np.int64).reshape((height, width))
    occ = np.ascontiguousarray(arr > 10, dtype=np.uint8)
    angle = -1.0 * _quaternion_yaw(info.origin.orientation)
    world = (float(info.resolution), angle, float(info.origin.position.x), float(info.origin.position.y),
             float(np.sin(angle)), float(np.cos(angle)))
    return occ, world


def trig_eval(x) -> np.ndarray:
    """(sin, cos) pairs [n, 2] that the BL and RM casts use for headings x when no trig override
    is set: the floats nearest to the exact values, computed on the device (rlc_trig_eval)."""
    x = np.ascontiguousarray(x, np.float32).reshape(-1)
    out = np.empty((x.size, 2), np.float32)
    call("rlc_trig_eval", x.ctypes.data, out.ctypes.data, x.size, 0, None)
    return out


# ---------------------------------------------------------------- PyOMap
class PyOMap:
    """Occupancy grid (OMap, RangeLib.h:121-322; PyOMap, RangeLibc.pyx:130-197).

    PyOMap(width, height)          empty map
    PyOMap(path[, threshold])      PNG: grey (0.229 B + 0.587 G + 0.114 R, as the
                                   reference reads its channels) < threshold is occupied
    PyOMap(ndarray)                bool array indexed [row, col]; grid[x][y] = arr[y, x]
    PyOMap(occupancy_grid_msg)     any object shaped like nav_msgs/OccupancyGrid:
                                   cells > 10 are occupied, world parameters from info
    """

    def __init__(self, arg1, arg2=None):
        self._error = False
        self.fn = ""   # the PNG's path, as OMap::fn
        world = (1.0, 0.0, 0.0, 0.0, 0.0, 1.0)
        if arg1 is not None and arg2 is not None and isinstance(arg1, (int, np.integer)):
            occ = np.zeros((int(arg1), int(arg2)), np.uint8)
        elif arg1 is not None and arg2 is not None:
            self.fn = str(arg1)
            occ = self._from_png(str(arg1), float(arg2))
        elif isinstance(arg1, np.ndarray):
            occ = np.ascontiguousarray((arg1 != 0).T, dtype=np.uint8)
        elif hasattr(arg1, "info") and hasattr(arg1, "data"):
            occ, world = occupancy_grid_parts(arg1)
        elif isinstance(arg1, str):
            self.fn = arg1
            occ = self._from_png(arg1, 128.0)
        else:
            print("Failed to construct PyOMap, check argument types.")
            occ = np.zeros((1, 1), np.uint8)
        if occ.size == 0:
            occ = np.zeros((1, 1), np.uint8)
            self._error = True
        self._occ = np.ascontiguousarray(occ, dtype=np.uint8)
        self.world = tuple(float(np.float32(v)) for v in world)
        h = C.c_void_p()
        W, H = self._occ.shape
        call("rlc_map_create", self._occ.ctypes.data_as(_lib._u8p), W, H, C.byref(h))
        self._h = h
        call("rlc_map_set_world", self._h, *self.world)

    def _from_png(self, path: str, threshold: float) -> np.ndarray:
        try:
            return png_occupancy(path, threshold)
        except _lib.RangeLibError as e:   # the reference prints the decoder's error and flags the map
            print(f"ERROR: {e}")
            self._error = True
            return np.zeros((0, 0), np.uint8)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _lib._lib is not None:
            _lib._lib.rlc_map_destroy(h)
            self._h = None

    @property
    def handle(self):
        return self._h

    def set_world(self, scale: float, angle: float, origin_x: float, origin_y: float,
                  sin_angle: float | None = None, cos_angle: float | None = None) -> None:
        """World parameters of the ROS conversion (the OMap fields the OccupancyGrid path sets).

        Methods copy them when they are created, like the reference's by-value OMap."""
        if sin_angle is None:
            sin_angle = float(np.sin(angle))
        if cos_angle is None:
            cos_angle = float(np.cos(angle))
        self.world = tuple(float(np.float32(v)) for v in (scale, angle, origin_x, origin_y, sin_angle, cos_angle))
        call("rlc_map_set_world", self._h, *self.world)

    @property
    def occupancy(self) -> np.ndarray:
        """grid[x][y] as a uint8 array of shape (width, height)."""
        return self._occ

    def save(self, fn) -> bool:
        """PNG with white = free, black = occupied (OMap::save, RangeLib.h:263-291); False on
        success, like the reference's encoder status."""
        W, H = self._occ.shape
        rc = lib().rlc_png_save_occupancy(fn.encode() if isinstance(fn, str) else bytes(fn), self._occ.ctypes.data, W, H)
        if rc != _lib.RLC_OK:
            print(f"encoder error {rc}: {lib().rlc_last_error().decode()}")
        return rc != _lib.RLC_OK

    def isOccupied(self, x: int, y: int) -> bool:
        return bool(self._occ[x, y])

    def error(self) -> bool:
        return self._error

    def width(self) -> int:
        return int(self._occ.shape[0])

    def height(self) -> int:
        return int(self._occ.shape[1])


# ---------------------------------------------------------------- methods
class _RangeMethod:
    _kind = None

    def __init__(self, Map: PyOMap, max_range: float, theta_disc: int = 0, *, _trig=None):
        self.map = Map
        self.max_range = float(np.float32(max_range))
        self.theta_disc = int(theta_disc)
        h = C.c_void_p()
        if _trig is not None:
            cos_t = np.ascontiguousarray(_trig[0], np.float32)
            sin_t = np.ascontiguousarray(_trig[1], np.float32)
            call("rlc_method_create_cddt_trig", Map.handle, self._kind, self.max_range, self.theta_disc,
                 cos_t.ctypes.data_as(_lib._f32p), sin_t.ctypes.data_as(_lib._f32p), C.byref(h))
        else:
            call("rlc_method_create", Map.handle, self._kind, self.max_range, self.theta_disc, C.byref(h))
        self._h = h
        self._table_width = 0

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _lib._lib is not None:
            _lib._lib.rlc_method_destroy(h)
            self._h = None

    @property
    def handle(self):
        return self._h

    # RangeMethod::calc_range -- one ray in grid space (no world transform)
    def calc_range(self, x: float, y: float, heading: float) -> float:
        out = C.c_float()
        call("rlc_calc_range", self._h, float(x), float(y), float(heading), C.byref(out))
        return out.value

    def calc_range_many(self, ins, outs) -> None:
        F = _lib.fast()
        if F is not None:   # numpy buffers straight to the C ABI; -1: not a plain buffer, check below
            rc = F.calc_range_many(self._h.value, ins, outs)
            if rc != -1:
                return _lib.check(rc)
        pi, di = _arg(ins, np.float32, 2, "ins")
        po, do = _arg(outs, np.float32, 1, "outs")
        flags, stream = _flags_stream([di, do], ins)
        n = outs.shape[0]
        if n and ins.shape[0] < n:
            raise ValueError("ins has fewer rows than outs")
        call("rlc_calc_range_many", self._h, pi, po, n, flags, stream)

    def calc_range_repeat_angles(self, ins, angles, outs) -> None:
        F = _lib.fast()
        if F is not None:
            rc = F.repeat_angles(self._h.value, ins, angles, outs)
            if rc != -1:
                return _lib.check(rc)
        pi, di = _arg(ins, np.float32, 2, "ins")
        pa, da = _arg(angles, np.float32, 1, "angles")
        po, do = _arg(outs, np.float32, 1, "outs")
        flags, stream = _flags_stream([di, da, do], ins)
        n, na = ins.shape[0], angles.shape[0]
        if outs.shape[0] < n * na:
            raise ValueError(f"outs needs {n * na} entries")
        call("rlc_calc_range_repeat_angles", self._h, pi, pa, po, n, na, flags, stream)

    def set_sensor_model(self, table) -> None:
        if not isinstance(table, np.ndarray) or table.dtype != np.float64 or table.ndim != 2:
            raise ValueError("Buffer dtype mismatch: the sensor model is a 2-D float64 array")
        if not table.shape[0] == table.shape[1]:
            print("Sensor model must have equal matrix dimensions, failing!")
            return
        t = np.ascontiguousarray(table)
        call("rlc_set_sensor_model", self._h, t.ctypes.data_as(_lib._f64p), t.shape[0])
        self._table_width = t.shape[0]

    def eval_sensor_model(self, observation, ranges, outs, num_rays: int, num_particles: int) -> None:
        F = _lib.fast()
        if F is not None:
            rc = F.eval_sensor_model(self._h.value, observation, ranges, outs, num_rays, num_particles)
            if rc != -1:
                return _lib.check(rc)
        po, do = _arg(observation, np.float32, 1, "observation")
        pr, dr = _arg(ranges, np.float32, 1, "ranges")
        pw, dw = _arg(outs, np.float64, 1, "outs")
        flags, stream = _flags_stream([do, dr, dw], observation)
        if observation.shape[0] < num_rays or ranges.shape[0] < num_rays * num_particles or outs.shape[0] < num_particles:
            raise ValueError("array shorter than num_rays / num_particles")
        call("rlc_eval_sensor_model", self._h, po, pr, pw, int(num_rays), int(num_particles), flags, stream)

    def calc_range_repeat_angles_eval_sensor_model(self, ins, angles, obs, weights) -> None:
        F = _lib.fast()
        if F is not None:
            rc = F.fused(self._h.value, ins, angles, obs, weights)
            if rc != -1:
                return _lib.check(rc)
        pi, di = _arg(ins, np.float32, 2, "ins")
        pa, da = _arg(angles, np.float32, 1, "angles")
        po, do = _arg(obs, np.float32, 1, "obs")
        pw, dw = _arg(weights, np.float64, 1, "weights")
        flags, stream = _flags_stream([di, da, do, dw], ins)
        n, na = ins.shape[0], angles.shape[0]
        if obs.shape[0] < na or weights.shape[0] < n:
            raise ValueError("obs needs one entry per angle and weights one per particle")
        call("rlc_calc_range_repeat_angles_eval_sensor_model", self._h, pi, pa, po, pw, n, na, flags, stream)

    def saveTrace(self, path) -> float:
        print("WARNING: trace map not generated, must compile with trace support enabled.")
        return 0.0

    # ---- extras (no reference counterpart) ----
    def device_flags(self) -> int:
        f = C.c_uint()
        call("rlc_method_device_flags", self._h, C.byref(f))
        return f.value

    def set_trig_override(self, trig) -> None:
        """Parity mode: per-ray (cos, sin) used by the next BL/RM queries (None restores sincosf)."""
        if trig is None:
            call("rlc_method_set_trig_override", self._h, None, 0)
            return
        t = np.ascontiguousarray(trig, np.float32).reshape(-1, 2)
        self._trig = t
        call("rlc_method_set_trig_override", self._h, t.ctypes.data_as(_lib._f32p), t.shape[0])

    def count_steps(self, ins, angles) -> int:
        """Total march steps of the repeat-angle rays (RM: DT reads; BL: cells tested)."""
        pi, di = _arg(ins, np.float32, 2, "ins")
        pa, da = _arg(angles, np.float32, 1, "angles")
        flags, _ = _flags_stream([di, da], ins)
        tot = C.c_int64()
        call("rlc_count_steps", self._h, pi, pa, ins.shape[0], angles.shape[0], flags, C.byref(tot))
        return tot.value

    def set_schedule(self, dt_layout: int = 0, fused_block: int = 0, prefetch: int = 0, tile: int = 0) -> None:
        """dt_layout 0 linear / 1 tiled / 2 compact 16-bit / 4 per-cell step map / 5 step map with
        equal-step runs (a ray beside a wall skips its repeated steps exactly) / 3 beam-major update
        with staged 8-bit windows (-1: autotune on the next fused call), threads per block of the fused kernel
        (0 keeps it), prefetch (RM: 0 plain / 1 prefetching march; CDDT: 0 binary / 1 warp-cooperative /
        2 sector bin search), particles per tile (0 automatic; for layout 3 the particle
        chunks per beam).  Results do not depend on the schedule."""
        call("rlc_method_set_schedule", self._h, int(dt_layout), int(fused_block), int(prefetch), int(tile))

    def schedule(self):
        """(dt_layout, fused_block, prefetch, tile)"""
        a, b, c, d = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        call("rlc_method_get_schedule", self._h, C.byref(a), C.byref(b), C.byref(c), C.byref(d))
        return a.value, b.value, c.value, d.value

    def autotune(self, ins, angles, obs, weights, flush_l2: bool = False) -> None:
        """Time the schedule candidates on this workload (CUDA tensors) and keep the fastest;
        flush_l2 writes twice the L2 size before every timed launch (maps that leave L2 between
        updates)."""
        ptrs = [_arg(a, dt, nd, nm) for a, dt, nd, nm in ((ins, np.float32, 2, "ins"), (angles, np.float32, 1, "angles"),
                                                          (obs, np.float32, 1, "obs"), (weights, np.float64, 1, "weights"))]
        if not all(d for _, d in ptrs):
            raise ValueError("autotune takes CUDA tensors")
        call("rlc_method_autotune_ex", self._h, *[p for p, _ in ptrs], ins.shape[0], angles.shape[0],
             _lib.RLC_TUNE_FLUSH_L2 if flush_l2 else 0, _stream_of(ins))

    def autotune_results(self):
        """Candidates of the last autotune: list of ((dt_layout, fused_block, prefetch, tile),
        first-stage median ms, final median ms or None)."""
        n = C.c_int()
        call("rlc_method_autotune_results", self._h, 0, C.byref(n), None, None)
        sched = np.zeros((max(n.value, 1), 4), np.int32)
        ms = np.zeros((max(n.value, 1), 2), np.float32)
        call("rlc_method_autotune_results", self._h, n.value, C.byref(n), sched.ctypes.data, ms.ctypes.data)
        return [(tuple(int(v) for v in sched[i]), float(ms[i, 0]), float(ms[i, 1]) if ms[i, 1] > 0 else None)
                for i in range(n.value)]


class PyBresenhamsLine(_RangeMethod):
    """BresenhamsLine (RangeLib.h:691-772; RangeLibc.pyx:200-225)."""
    _kind = _lib.RLC_BL

    def __init__(self, Map: PyOMap, max_range: float):
        super().__init__(Map, max_range)


class PyRayMarching(_RangeMethod):
    """RayMarching (RangeLib.h:922-969; RangeLibc.pyx:227-251)."""
    _kind = _lib.RLC_RM

    def __init__(self, Map: PyOMap, max_range: float):
        super().__init__(Map, max_range)


class PyCDDTCast(_RangeMethod):
    """CDDTCast (RangeLib.h:971-1770; RangeLibc.pyx:253-287); the table is built on the GPU."""
    _kind = _lib.RLC_CDDT

    def __init__(self, Map: PyOMap, max_range: float, theta_disc: int, *, trig=None):
        super().__init__(Map, max_range, theta_disc, _trig=trig)

    def prune(self, max_range: float = -1.0) -> None:
        call("rlc_cddt_prune", self._h, self.max_range if max_range < 0.0 else float(max_range))

    def table(self):
        """(widths[td], translations[td], bin_len[num_bins], zeros) -- compressed_lut in CSR form."""
        nb, nz = C.c_int64(), C.c_int64()
        call("rlc_cddt_table_size", self._h, C.byref(nb), C.byref(nz))
        widths = np.empty(self.theta_disc, np.int32)
        trans = np.empty(self.theta_disc, np.float32)
        bin_len = np.empty(nb.value, np.int64)
        zeros = np.empty(max(nz.value, 1), np.float32)
        call("rlc_cddt_table_export", self._h, widths.ctypes.data_as(_lib._i32p), trans.ctypes.data_as(_lib._f32p),
             bin_len.ctypes.data_as(_lib._i64p), zeros.ctypes.data_as(_lib._f32p))
        return widths, trans, bin_len, zeros[: nz.value]

    def load_table(self, trans, bin_len, zeros) -> None:
        trans = np.ascontiguousarray(trans, np.float32)
        bin_len = np.ascontiguousarray(bin_len, np.int64)
        zeros = np.ascontiguousarray(zeros, np.float32)
        call("rlc_cddt_table_load", self._h, trans.ctypes.data_as(_lib._f32p), bin_len.ctypes.data_as(_lib._i64p),
             zeros.ctypes.data_as(_lib._f32p), len(zeros))

    def serialize_json(self, precision: int = 9) -> str:
        """The table as CDDTCast::serializeJson writes it (RangeLib.h:1690-1735); 9 significant
        digits by default so that load_json restores it exactly (7 gives the reference's text)."""
        widths, trans, bin_len, zeros = self.table()
        return cddt_json_dumps(self.theta_disc, self.max_range, trans, widths, bin_len, zeros,
                               self.map.occupancy, self.map.fn, precision)

    def load_json(self, text: str) -> None:
        """Replace the table by one serialised for the same map and theta_disc (by serialize_json
        or the reference's serializeJson)."""
        d = cddt_json_loads(text)
        widths = self.table()[0]
        if d["theta_disc"] != self.theta_disc or not np.array_equal(d["widths"], widths):
            raise ValueError("the serialised table has another theta_discretization or other slice widths")
        if d["occ"].shape != self.map.occupancy.shape:
            raise ValueError("the serialised table was built for a map of another size")
        self.load_table(d["trans"], d["bin_len"], d["zeros"])

    @classmethod
    def from_json(cls, text: str, *, trig=None) -> "PyCDDTCast":
        """A CDDTCast over the document's own map and max_range, with the document's table."""
        d = cddt_json_loads(text)
        omap = PyOMap(np.ascontiguousarray(d["occ"].T))
        omap.fn = d["path"]
        m = cls(omap, d["max_range"], d["theta_disc"], trig=trig)
        m.load_table(d["trans"], d["bin_len"], d["zeros"])
        return m

    def calc_range_pair(self, x: float, y: float, heading: float):
        """CDDTCast::calc_range_pair (RangeLib.h:1521-1615): (range at heading, range at heading + pi)."""
        r, ri = C.c_float(), C.c_float()
        call("rlc_cddt_calc_range_pair", self._h, float(x), float(y), float(heading), C.byref(r), C.byref(ri))
        return r.value, ri.value

    def calc_range_many_radial_optimized(self, num_rays: int, min_angle: float, max_angle: float, ins, outs) -> None:
        """CDDTCast::calc_range_many_radial_optimized (RangeLib.h:616-676; RangeLibc.pyx:275-277):
        world-frame poses ins[n, 3], outs[n * num_rays]; the first num_rays / 3 beams are cast in
        pairs with the beam pi further on.  Positions the reference leaves unwritten keep their values."""
        pi, di = _arg(ins, np.float32, 2, "ins")
        po, do = _arg(outs, np.float32, 1, "outs")
        flags, stream = _flags_stream([di, do], ins)
        n = ins.shape[0]
        if outs.shape[0] != n * int(num_rays):
            raise ValueError("outs must hold len(ins) * num_rays ranges")
        call("rlc_cddt_calc_range_many_radial", self._h, pi, po, n, int(num_rays), float(min_angle), float(max_angle),
             flags, stream)


class PyGiantLUTCast(_RangeMethod):
    """GiantLUTCast (RangeLib.h:1772-1904; RangeLibc.pyx:288-312): a width x height x td table of
    16-bit ranges, built on the GPU by one ray march from every cell corner at every angle bin;
    each query is one table read."""
    _kind = _lib.RLC_GLT

    def __init__(self, Map: PyOMap, max_range: float, theta_disc: int, *, trig=None):
        super().__init__(Map, max_range, theta_disc, _trig=trig)

    def lut(self) -> np.ndarray:
        """The table as uint16 [width, height, td] (giant_lut[x][y][i])."""
        w, h = self.map.width(), self.map.height()
        out = np.empty((w, h, self.theta_disc), np.uint16)
        call("rlc_glt_table", self._h, out.ctypes.data_as(C.POINTER(C.c_uint16)))
        return out


class PyRayMarchingGPU(_RangeMethod):
    """RayMarchingGPU (RangeLib.h:774-920; RangeLibc.pyx:314-340)."""
    _kind = _lib.RLC_RMGPU

    def __init__(self, Map: PyOMap, max_range: float):
        super().__init__(Map, max_range)


class PyNull:
    """Call-overhead probe of the reference (RangeLibc.pyx:342-351)."""

    def __init__(self, Map, max_range, theta_disc):
        pass

    def calc_range(self, x, y, heading):
        return x + y + heading

    def calc_range_many(self, ins, outs):
        a = ins[0, 0]
        b = outs[0]
        c = outs.shape[0]
        return a, b, c


# ---------------------------------------------------------------- host buffers
def set_host_path(mode: str = "auto") -> None:
    """'auto': host (numpy) buffers are read and written in place by the kernels where the GPU
    accesses host memory coherently (Grace + Blackwell, NVLink-C2C), else staged; 'staged':
    always staged through device memory.  Process-wide."""
    call("rlc_set_host_path", {"auto": _lib.RLC_HOST_AUTO, "staged": _lib.RLC_HOST_STAGED}[mode])


def host_path_direct() -> bool:
    """True if host-buffer calls on the current device run in place."""
    v = C.c_int()
    call("rlc_host_path", C.byref(v))
    return bool(v.value)


# ---------------------------------------------------------------- batch
class PyFilterBatch:
    """Many particle filters updated by one persistent launch, replayed as a CUDA graph.

    filters: list of (method, ins, angles, obs, weights[, ranges]) with CUDA tensors;
    every method needs its sensor model set.  run() queues the whole update on
    the current stream.  No reference counterpart.
    """

    def __init__(self, filters, block: int = 0):
        self._keep = []
        descs = (_lib.FilterDesc * len(filters))()
        for i, f in enumerate(filters):
            method, ins, angles, obs, weights = f[:5]
            ranges = f[5] if len(f) > 5 else None
            for a, dt, nd, nm in ((ins, np.float32, 2, "ins"), (angles, np.float32, 1, "angles"),
                                  (obs, np.float32, 1, "obs"), (weights, np.float64, 1, "weights")):
                if not _arg(a, dt, nd, nm)[1]:
                    raise ValueError("batched filters take CUDA tensors")
            d = descs[i]
            d.method = method.handle
            d.ins, d.angles, d.obs, d.weights = ins.data_ptr(), angles.data_ptr(), obs.data_ptr(), weights.data_ptr()
            d.ranges = ranges.data_ptr() if ranges is not None else None
            d.n_particles, d.n_angles = ins.shape[0], angles.shape[0]
            self._keep.append((method, ins, angles, obs, weights, ranges))
        h = C.c_void_p()
        call("rlc_batch_create", descs, len(filters), int(block), C.byref(h))
        self._h = h
        self._device = filters[0][1].device

    def run(self) -> None:
        call("rlc_batch_run", self._h, _stream_of(self._keep[0][1]))

    def set_schedule(self, dt_layout: int = 0, prefetch: int = 0, block: int = 0, tile: int = 0) -> None:
        call("rlc_batch_set_schedule", self._h, int(dt_layout), int(prefetch), int(block), int(tile))

    def set_product_mode(self, separate: bool) -> None:
        """Per-particle products inside the persistent kernel (False) or in a second launch (True)."""
        call("rlc_batch_set_product_mode", self._h, 1 if separate else 0)

    def product_mode(self) -> str:
        v = C.c_int()
        call("rlc_batch_get_product_mode", self._h, C.byref(v))
        return "separate" if v.value else "overlapped"

    def schedule(self):
        """(dt_layout, prefetch, block, tile)"""
        v = [C.c_int() for _ in range(4)]
        call("rlc_batch_get_schedule", self._h, *[C.byref(x) for x in v])
        return tuple(x.value for x in v)

    def autotune(self) -> None:
        """Run the batch under each schedule candidate and keep the fastest (outputs are rewritten)."""
        call("rlc_batch_autotune", self._h, _stream_of(self._keep[0][1]))

    def info(self):
        r, t = C.c_int64(), C.c_int64()
        call("rlc_batch_info", self._h, C.byref(r), C.byref(t))
        return r.value, t.value

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _lib._lib is not None:
            _lib._lib.rlc_batch_destroy(h)
            self._h = None


class PyLearnedRM:
    """Learned range surrogate of a ray-marching method's map (no reference counterpart).

    A Fourier-feature MLP (512 features, 4 x 256 GELU, BF16 weights, FP32 accumulation) is
    trained on the GPU, on rays the exact marcher casts, to predict the march parameter of a
    ray's hit cell.  calc_range_repeat_angles accepts a prediction whose cell is occupied and
    whose previous cell (one pixel back) is free, returns the reference's distance to that
    cell's corner, and recasts every other ray exactly.  Arrays are CUDA tensors.
    """

    def __init__(self, method, seed: int = 0):
        import torch  # noqa: F401
        h = C.c_void_p()
        call("rlc_learned_create", method.handle, int(seed), C.byref(h))
        self._h = h
        self.method = method
        self.n_params = int(lib().rlc_learned_param_count())

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _lib._lib is not None:
            _lib._lib.rlc_learned_destroy(h)
            self._h = None

    def train(self, steps: int, batch: int = 8192, lr: float = 1e-3, seed: int = 1) -> float:
        loss = C.c_float()
        call("rlc_learned_train", self._h, int(steps), int(batch), float(lr), int(seed), C.byref(loss), None)
        return loss.value

    def sample_rays(self, n: int, first_id: int = 0, seed: int = 7):
        """(xyt [n, 3] grid-frame rays, t [n] hit parameter, range [n] exact range) from the exact marcher."""
        import torch
        dev = torch.device("cuda", torch.cuda.current_device())
        xyt = torch.empty((n, 3), dtype=torch.float32, device=dev)
        t = torch.empty(n, dtype=torch.float32, device=dev)
        r = torch.empty(n, dtype=torch.float32, device=dev)
        call("rlc_learned_sample_rays", self._h, int(first_id), int(seed), int(n), xyt.data_ptr(), t.data_ptr(),
             r.data_ptr(), _stream_of(xyt))
        return xyt, t, r

    def predict(self, xyt, layered: bool = False):
        """Predicted hit parameter t of grid-frame rays xyt [n, 3] (CUDA): the fused forward kernel,
        or with layered=True the training path's layer-by-layer GEMMs (bit-identical)."""
        import torch
        out = torch.empty(xyt.shape[0], dtype=torch.float32, device=xyt.device)
        call("rlc_learned_predict_layered" if layered else "rlc_learned_predict", self._h, xyt.data_ptr(),
             int(xyt.shape[0]), out.data_ptr(), _stream_of(xyt))
        return out

    def features(self, xyt):
        import torch
        out = torch.empty((xyt.shape[0], 512), dtype=torch.bfloat16, device=xyt.device)
        call("rlc_learned_features", self._h, xyt.data_ptr(), int(xyt.shape[0]), out.data_ptr())
        return out

    def gradients(self, xyt, t):
        g = np.empty(self.n_params, np.float32)
        loss = C.c_float()
        call("rlc_learned_gradients", self._h, xyt.data_ptr(), t.data_ptr(), int(xyt.shape[0]),
             g.ctypes.data_as(_lib._f32p), C.byref(loss))
        return g, loss.value

    def params(self) -> np.ndarray:
        p = np.empty(self.n_params, np.float32)
        call("rlc_learned_get_params", self._h, p.ctypes.data_as(_lib._f32p))
        return p

    def set_params(self, p) -> None:
        p = np.ascontiguousarray(p, np.float32)
        call("rlc_learned_set_params", self._h, p.ctypes.data_as(_lib._f32p))

    def calc_range_repeat_angles(self, ins, angles, outs, accepted=None) -> int:
        """World-frame particles x beams (like PyRayMarching.calc_range_repeat_angles); returns
        the number of rays recast exactly."""
        nrec = C.c_int64()
        call("rlc_learned_calc_range_repeat_angles", self._h, ins.data_ptr(), angles.data_ptr(), outs.data_ptr(),
             int(ins.shape[0]), int(angles.shape[0]), None if accepted is None else accepted.data_ptr(),
             C.byref(nrec), _stream_of(ins))
        return nrec.value


def tc_gemm(a, b, M, N, K, a_t=False, b_t=False):
    """C = A . B^T on the tensor cores (bf16 CUDA tensors in, fp32 out); test hook."""
    import torch
    c = torch.empty((M, N), dtype=torch.float32, device=a.device)
    call("rlc_tc_gemm", a.data_ptr(), b.data_ptr(), c.data_ptr(), int(M), int(N), int(K), int(a_t), int(b_t),
         _stream_of(a))
    return c


def device_count() -> int:
    return lib().rlc_device_count()


def library_path() -> str:
    return _lib.library_path()


__all__ = [
    "PyOMap", "PyBresenhamsLine", "PyRayMarching", "PyCDDTCast", "PyGiantLUTCast", "PyRayMarchingGPU", "PyNull",
    "PyFilterBatch", "set_host_path", "host_path_direct", "USE_CACHED_TRIG", "USE_ALTERNATE_MOD", "USE_CACHED_CONSTANTS", "USE_FAST_ROUND",
    "NO_INLINE", "USE_LRU_CACHE", "LRU_CACHE_SIZE", "SHOULD_USE_CUDA",
]

if __name__ == "__main__":  # pragma: no cover
    print(library_path(), device_count(), file=sys.stderr)
