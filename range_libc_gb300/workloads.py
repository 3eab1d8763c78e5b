"""Seeded synthetic workloads for the ray-casting path (maps, poses, sensor tables).

All maps are ``uint8`` occupancy grids ``occ[x, y]`` of shape ``(width, height)``
-- the reference's ``OMap::grid[x][y]`` layout.  Randomness is
``numpy.random.default_rng(seed)`` (PCG64, stable across numpy versions).

Axis convention of the world-frame APIs (RangeLib.h:439-480): a world pose
``(xw, yw, theta)`` lands on grid cell ``x = (yw - oy)/s`` (first index) and
``y = (xw - ox)/s`` (second index), because the reference calls
``calc_range(y, x, theta)`` after its transform.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np


# --------------------------------------------------------------------------
# maps
# --------------------------------------------------------------------------
def rect_disk_map(side: int, seed: int, n_rects: int | None = None, n_disks: int | None = None) -> np.ndarray:
    """Square map with a 1-px border wall, filled axis-aligned rectangles
    (sides U[5, 60]) and filled disks (radius U[3, 25]); shape centres are
    uniform over the map and clipped at its edge.  At side 512 the counts are
    40 rectangles and 20 disks; larger sides scale the counts by area."""
    rng = np.random.default_rng(seed)
    scale = (side / 512.0) ** 2
    n_rects = int(round(40 * scale)) if n_rects is None else n_rects
    n_disks = int(round(20 * scale)) if n_disks is None else n_disks
    occ = np.zeros((side, side), np.uint8)
    occ[0, :] = occ[-1, :] = occ[:, 0] = occ[:, -1] = 1
    for _ in range(n_rects):
        w, h = rng.integers(5, 61, size=2)
        cx, cy = rng.uniform(0, side, size=2)
        x0, y0 = int(cx - w / 2), int(cy - h / 2)
        occ[max(x0, 0):max(min(x0 + w, side), 0), max(y0, 0):max(min(y0 + h, side), 0)] = 1
    for _ in range(n_disks):
        r = rng.uniform(3, 25)
        cx, cy = rng.uniform(0, side, size=2)
        x0, x1 = max(int(cx - r) - 1, 0), min(int(cx + r) + 2, side)
        y0, y1 = max(int(cy - r) - 1, 0), min(int(cy + r) + 2, side)
        if x0 >= x1 or y0 >= y1:
            continue
        xs = np.arange(x0, x1)[:, None] + 0.5
        ys = np.arange(y0, y1)[None, :] + 0.5
        occ[x0:x1, y0:y1] |= ((xs - cx) ** 2 + (ys - cy) ** 2 <= r * r).astype(np.uint8)
    return occ


def corridor_map(side: int, seed: int) -> np.ndarray:
    """Rectilinear rooms 40-200 px wide made by recursive splits; every
    splitting wall is 2-4 px thick with one door gap of 8-16 px."""
    rng = np.random.default_rng(seed)
    occ = np.zeros((side, side), np.uint8)
    t = 3
    occ[:t, :] = occ[-t:, :] = occ[:, :t] = occ[:, -t:] = 1
    stack = [(t, t, side - t, side - t)]          # free interior [x0, x1) x [y0, y1)
    while stack:
        x0, y0, x1, y1 = stack.pop()
        w, h = x1 - x0, y1 - y0
        axes = [a for a, ext in ((0, w), (1, h)) if ext > 200]
        if not axes:
            continue
        axis = axes[int(rng.integers(len(axes)))] if len(axes) > 1 else axes[0]
        lo_, hi_ = (x0, x1) if axis == 0 else (y0, y1)
        th = int(rng.integers(2, 5))
        lo = lo_ + 40
        hi = hi_ - 40 - th
        if hi <= lo:
            continue
        cut = int(rng.integers(lo, hi + 1))
        door = int(rng.integers(8, 17))
        if axis == 0:
            occ[cut:cut + th, y0:y1] = 1
            d0 = int(rng.integers(y0, max(y0 + 1, y1 - door)))
            occ[cut:cut + th, d0:d0 + door] = 0
            stack += [(x0, y0, cut, y1), (cut + th, y0, x1, y1)]
        else:
            occ[x0:x1, cut:cut + th] = 1
            d0 = int(rng.integers(x0, max(x0 + 1, x1 - door)))
            occ[d0:d0 + door, cut:cut + th] = 0
            stack += [(x0, y0, x1, cut), (x0, cut + th, x1, y1)]
    return occ


def free_cell_queries(occ: np.ndarray, n: int, seed: int) -> np.ndarray:
    """``n`` float32 queries (x, y, theta): a uniformly drawn free cell index
    plus U[0, 1) in each axis, theta ~ U[0, 2*pi)."""
    rng = np.random.default_rng(seed)
    free = np.flatnonzero(occ.reshape(-1) == 0)
    pick = free[rng.integers(0, len(free), size=n)]
    H = occ.shape[1]
    q = np.empty((n, 3), np.float32)
    q[:, 0] = (pick // H) + rng.random(n)
    q[:, 1] = (pick % H) + rng.random(n)
    q[:, 2] = rng.uniform(0.0, 2.0 * math.pi, size=n)
    return q


def grid_to_world(gx, gy, world):
    """Grid cell coordinates (first index, second index) -> world (xw, yw),
    inverting RangeLib.h:468-473 for world angle 0 and 90-degree multiples."""
    s, _a, ox, oy, sa, ca = world
    # calc_range(y, x): first grid index = rotated y, second = rotated x
    x_rot, y_rot = gy, gx
    # undo the rotation [ca -sa; sa ca]
    xr = ca * x_rot + sa * y_rot
    yr = -sa * x_rot + ca * y_rot
    return xr * s + ox, yr * s + oy


def laser_angles(m: int, fov: float = 1.5 * math.pi) -> np.ndarray:
    return np.linspace(-fov / 2, fov / 2, m).astype(np.float32)


def sensor_table(K: int, sigma_hit: float = 8.0, lam_short: float = 0.01,
                 z_hit: float = 0.75, z_short: float = 0.01, z_max: float = 0.07,
                 z_rand: float = 0.12) -> np.ndarray:
    """K x K float64 table[r, d]: r = observed range bin, d = expected range
    bin.  Mixture of a Gaussian hit term, a short exponential, a max-range
    spike and a uniform term; every column sums to 1."""
    r = np.arange(K, dtype=np.float64)[:, None]
    d = np.arange(K, dtype=np.float64)[None, :]
    hit = np.exp(-0.5 * ((r - d) / sigma_hit) ** 2) / (sigma_hit * math.sqrt(2 * math.pi))
    short = np.where(r < d, lam_short * np.exp(-lam_short * r), 0.0)
    mx = (r == K - 1).astype(np.float64)
    table = z_hit * hit + z_short * short + z_max * mx + z_rand / K
    return table / table.sum(axis=0, keepdims=True)


def _cast_occupancy(occ: np.ndarray, x: float, y: float, heading: float, max_range: float) -> float:
    """Fine-stepped cast on the occupancy grid, used only to synthesise observations."""
    c, s = math.cos(heading), math.sin(heading)
    W, H = occ.shape
    t = 0.0
    while t < max_range:
        px, py = int(math.floor(x + c * t)), int(math.floor(y + s * t))
        if not (0 <= px < W and 0 <= py < H):
            return max_range
        if occ[px, py]:
            return t
        t += 0.1
    return max_range


# --------------------------------------------------------------------------
# named workloads
# --------------------------------------------------------------------------
@dataclass
class Workload:
    name: str
    occ: np.ndarray
    max_range: float
    world: tuple
    ins: np.ndarray                 # [N, 3] float32 queries / particles
    angles: np.ndarray | None = None
    obs: np.ndarray | None = None
    table: np.ndarray | None = None
    td: int | None = None


def rect_disk_queries(side=512, n=10_000, max_range=300.0, seed=1000) -> Workload:
    """Plain calc_range_many on a rectangles-and-disks map (identity world)."""
    occ = rect_disk_map(side, seed)
    ins = free_cell_queries(occ, n, seed + 1)
    # identity world: calc_range(y, x) swaps, so hand the swapped pose to the
    # world API to query grid cell (ins[:,0], ins[:,1])
    q = ins.copy()
    q[:, 0], q[:, 1] = ins[:, 1], ins[:, 0]
    return Workload(f"rect_disk_{side}_q{n}", occ, max_range, (1.0, 0.0, 0.0, 0.0, 0.0, 1.0), q)


def particle_filter_step(side=2048, n_particles=4000, n_beams=61, max_range_px=200.0,
                         scale=0.05, seed=2000, origin=(-12.5, -7.5)) -> Workload:
    """One particle-filter update on a corridor map at ``scale`` m/px:
    Gaussian particles (sigma 20 px, heading sigma 0.3 rad) about a free
    true pose, beams over 270 degrees, a K = int(max_range_px) + 1 sensor
    table and observations cast from the true pose plus N(0, 2 px) noise."""
    rng = np.random.default_rng(seed)
    occ = corridor_map(side, seed)
    world = (scale, 0.0, origin[0], origin[1], 0.0, 1.0)
    free = np.argwhere(occ == 0)
    # a true pose well inside the free space
    while True:
        gx, gy = free[rng.integers(len(free))] + 0.5
        if min(gx, gy, side - gx, side - gy) > 60:
            break
    theta_true = float(rng.uniform(0, 2 * math.pi))
    px = rng.normal(gx, 20.0, n_particles)
    py = rng.normal(gy, 20.0, n_particles)
    th = rng.normal(theta_true, 0.3, n_particles)
    xw, yw = grid_to_world(px, py, world)
    ins = np.stack([xw, yw, th], axis=1).astype(np.float32)
    angles = laser_angles(n_beams)
    K = int(max_range_px) + 1
    table = sensor_table(K)
    # observations: cast from the true pose in the grid frame of calc_range(y, x, th)
    rc = float(np.float32(-0.0 - 3.0 * math.pi / 2.0))
    gth = -theta_true + rc
    obs_px = np.array([_cast_occupancy(occ, gx, gy, gth - float(a), max_range_px) for a in angles])
    obs = ((obs_px + rng.normal(0, 2.0, n_beams)) * scale).astype(np.float32)
    return Workload(f"corridor_{side}_pf{n_particles}x{n_beams}", occ, max_range_px, world, ins,
                    angles, obs, table)


def cddt_queries(side=2048, n=1_000_000, td=108, max_range=300.0, seed=3000) -> Workload:
    occ = rect_disk_map(side, seed)
    ins = free_cell_queries(occ, n, seed + 1)
    q = ins.copy()
    q[:, 0], q[:, 1] = ins[:, 1], ins[:, 0]
    return Workload(f"cddt_{side}_td{td}_q{n}", occ, max_range, (1.0, 0.0, 0.0, 0.0, 0.0, 1.0), q, td=td)


@dataclass
class FilterSpec:
    side: int
    n_particles: int
    n_beams: int
    max_range: float
    seed: int


def uneven_batch_specs(n_filters=32, seed=4000) -> list[FilterSpec]:
    """Sides from {512, 1024, 2048, 4096}, particles log-uniform over
    500-20,000, beams U{30..1081}, max_range U[100, 400] px."""
    rng = np.random.default_rng(seed)
    specs = []
    for f in range(n_filters):
        side = int(rng.choice([512, 1024, 2048, 4096]))
        n_p = int(round(math.exp(rng.uniform(math.log(500), math.log(20000)))))
        n_b = int(rng.integers(30, 1082))
        mr = float(rng.uniform(100, 400))
        specs.append(FilterSpec(side, n_p, n_b, mr, seed + f))
    return specs


def batch_filter(spec: FilterSpec) -> Workload:
    occ = rect_disk_map(spec.side, spec.seed)
    rng = np.random.default_rng(spec.seed + 7)
    ins = free_cell_queries(occ, spec.n_particles, spec.seed + 1)
    q = ins.copy()
    q[:, 0], q[:, 1] = ins[:, 1], ins[:, 0]
    angles = laser_angles(spec.n_beams)
    K = int(spec.max_range) + 1
    table = sensor_table(K)
    obs = rng.uniform(0, spec.max_range, spec.n_beams).astype(np.float32)
    return Workload(f"filter_{spec.side}_{spec.n_particles}x{spec.n_beams}", occ, spec.max_range,
                    (1.0, 0.0, 0.0, 0.0, 0.0, 1.0), q, angles, obs, table)
