"""PyOMap(OccupancyGrid): maps handed over as ROS nav_msgs/OccupancyGrid messages.

The reference builds such a map in its Cython module (RangeLibc.pyx:146-167): the message's
``data`` is reshaped to (height, width) rows, ``OMap(height, width)`` is created, and
``grid[x][y] = data[x, y] > 10`` with x the row; the world parameters are the message's
resolution, origin position and ``-yaw`` of its origin orientation (quaternion_to_angle,
RangeLibc.pyx:122-128, through ROS tf's euler_from_quaternion), with that angle's sine and
cosine.  ROS is not installed here, so the messages are plain objects of the same shape.
"""
import math
from types import SimpleNamespace as NS

import numpy as np
import pytest

from range_libc_gb300 import workloads as W


def _message(data_rows, resolution, origin, quat):
    height, width = data_rows.shape
    info = NS(width=width, height=height, resolution=resolution,
              origin=NS(position=NS(x=origin[0], y=origin[1], z=0.0),
                        orientation=NS(x=quat[0], y=quat[1], z=quat[2], w=quat[3])))
    return NS(info=info, data=[int(v) for v in data_rows.reshape(-1)])


def _rows(height=37, width=53, seed=5):
    """Message values -1 (unknown), 0, 10 (free) and 11, 100 (occupied), non-square."""
    rng = np.random.default_rng(seed)
    return rng.choice(np.array([-1, 0, 10, 11, 100]), size=(height, width), p=[0.2, 0.4, 0.1, 0.1, 0.2])


def _yaw_quat(yaw, scale=1.0):
    return (0.0, 0.0, scale * math.sin(yaw / 2.0), scale * math.cos(yaw / 2.0))


def test_occupancy_grid_parts_follow_the_ros_branch():
    from range_libc_gb300.range_libc import occupancy_grid_parts
    rows = _rows()
    msg = _message(rows, 0.05, (-3.25, 7.5), _yaw_quat(0.3))
    occ, world = occupancy_grid_parts(msg)
    assert occ.shape == (37, 53)                          # OMap(height, width): x runs over rows
    assert np.array_equal(occ, (rows > 10).astype(np.uint8))
    assert occ[rows == 10].sum() == 0 and occ[rows == 11].all() and occ[rows == -1].sum() == 0
    scale, angle, ox, oy, sa, ca = world
    assert scale == 0.05 and ox == -3.25 and oy == 7.5
    assert abs(angle + 0.3) < 1e-12                       # angle = -yaw
    assert sa == math.sin(angle) and ca == math.cos(angle)


def test_quaternion_yaw_matches_tf_for_scaled_and_degenerate_quaternions():
    from range_libc_gb300.range_libc import _quaternion_yaw
    for yaw in (-3.0, -1.2, 0.0, 0.3, 1.5707963, 2.9):
        q = NS(**dict(zip("xyzw", _yaw_quat(yaw))))
        assert abs(_quaternion_yaw(q) - yaw) < 1e-12
        q2 = NS(**dict(zip("xyzw", _yaw_quat(yaw, 2.5))))   # tf normalises the quaternion first
        assert abs(_quaternion_yaw(q2) - yaw) < 1e-12
    assert _quaternion_yaw(NS(x=0.0, y=0.0, z=0.0, w=0.0)) == 0.0   # tf: identity below eps
    # a pure rotation about x leaves yaw 0; about y by 90 degrees is gimbal lock (tf gives 0)
    assert abs(_quaternion_yaw(NS(x=math.sin(0.4), y=0.0, z=0.0, w=math.cos(0.4)))) < 1e-15
    assert _quaternion_yaw(NS(x=0.0, y=math.sqrt(0.5), z=0.0, w=math.sqrt(0.5))) == 0.0


def _world_poses(world, grid_pts, thetas):
    """World poses that land on the given calc_range-space points (first, second grid index):
    the inverse of the reference's scale, rotate, swap (RangeLib.h:468-475)."""
    s, _a, ox, oy, sa, ca = world
    g0, g1 = grid_pts[:, 0].astype(np.float64), grid_pts[:, 1].astype(np.float64)
    xr, yr = g1, g0
    x = ca * xr + sa * yr
    y = -sa * xr + ca * yr
    return np.stack([x * s + ox, y * s + oy, thetas], 1).astype(np.float32)


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["bl", "rm"])
def test_occupancy_grid_map_casts_like_the_oracle(rl, oracle_mod, kind):
    """A map built from a message equals the message's grid, carries the message's world frame,
    and BL/RM ranges through it (world-frame numpy_calc_range, parity mode) equal the oracle's
    with that world."""
    base = W.corridor_map(512, 31)[:300, :410]             # non-square rows x columns
    rows = np.where(base == 1, 100, 0)
    rows[::7, ::11] = -1                                   # unknown cells are free
    rows[5:9, 300:310] = 10                                 # 10 is still free
    rows[200:203, 17:19] = 11                               # 11 is occupied
    msg = _message(rows, 0.05, (-1.5, 2.25), _yaw_quat(-0.7))
    m = rl.PyOMap(msg)
    assert np.array_equal(m.occupancy, (rows > 10).astype(np.uint8))
    world = m.world
    assert abs(world[1] - np.float32(0.7)) < 1e-6
    q_grid = W.free_cell_queries(m.occupancy, 4000, 32)
    ins = _world_poses(world, q_grid[:, :2], q_grid[:, 2])
    meth = (rl.PyBresenhamsLine if kind == "bl" else rl.PyRayMarching)(m, 150.0)
    ref = oracle_mod.OracleMethod(m.occupancy, kind, 150.0, world=world)
    _, trig = oracle_mod.world_rays(world, ins)
    meth.set_trig_override(trig)
    out = np.empty(len(ins), np.float32)
    meth.calc_range_many(ins, out)
    exp = ref.calc_range_many(ins)
    assert np.array_equal(out.view(np.uint32), exp.view(np.uint32))
    assert np.mean(exp < np.float32(150.0 * 0.05)) > 0.5   # most rays meet a wall in range
