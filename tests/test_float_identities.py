"""Cheaper forms of the reference's float arithmetic that the kernels use, checked on CPU.

discretize_theta (RangeLib.h:1287-1340) compares a float heading with the double constants
M_2PI and M_PI and subtracts M_PI in double.  The kernels use float-only forms (the FP64 pipe
of GB300 is slow); these tests show the forms are identical for every float they are used on.
Bresenham's in-grid test is done with one floor conversion and an unsigned compare per axis;
a test shows it equals the reference's float comparisons for every float and width.
"""
import math

import numpy as np

K2PI = 6.28318530718            # RangeLib.h:61
M2PI_DOWN = np.float32(float.fromhex("0x1.921fb4p+2"))
MPI_UP = np.float32(float.fromhex("0x1.921fb6p+1"))
MPI_HI = np.float32(float.fromhex("0x1.921fb6p+1"))
MPI_LO = np.float32(float.fromhex("-0x1.777a5cp-24"))


def _next(f, toward):
    return np.nextafter(np.float32(f), np.float32(toward))


def test_range_comparisons():
    # (double)t > M_2PI  <=>  t > M2PI_DOWN : M2PI_DOWN <= M_2PI < next float
    assert float(M2PI_DOWN) <= K2PI < float(_next(M2PI_DOWN, 10))
    # (double)t >= M_PI  <=>  t >= MPI_UP : previous float < M_PI <= MPI_UP
    assert float(_next(MPI_UP, 0)) < math.pi <= float(MPI_UP)


def test_flip_subtraction_exhaustive():
    lo, hi = MPI_UP.view(np.uint32), M2PI_DOWN.view(np.uint32)
    t = np.arange(lo, hi + 1, dtype=np.uint32).view(np.float32)
    ref = (t.astype(np.float64) - math.pi).astype(np.float32)
    got = (t - MPI_HI) - MPI_LO
    assert got.dtype == np.float32 and len(t) == 8388608
    assert np.array_equal(ref.view(np.uint32), got.view(np.uint32))
    assert MPI_HI == np.float32(math.pi) and MPI_LO == np.float32(math.pi - float(MPI_HI))


def _f2i_rd(g):
    """__float2int_rd: floor, saturated to the int32 range (g is never NaN where it is used)."""
    f = np.floor(g.astype(np.float64))
    return np.clip(f, -2.0 ** 31, 2.0 ** 31 - 1).astype(np.int64)


def test_bresenham_in_grid_test():
    """Bresenham's in-grid test (RangeLib.h:696-769): the reference's `0 <= g && g < (float)W`
    equals `(unsigned)floor(g) < min(W, (float)W)` for every float g, with floor saturating like
    __float2int_rd, and floor(g) equals the reference's (int)g wherever the test passes.  Widths
    include ones whose float rounds down (2^24 + 1) and up (2^24 + 3)."""
    pats = np.arange(0, 2 ** 32, 4093, dtype=np.uint64).astype(np.uint32)
    g = pats.view(np.float32)
    extra = []
    for w in (1, 7, 1100, 2 ** 24 - 1, 2 ** 24, 2 ** 24 + 1, 2 ** 24 + 3, 2 ** 31 - 1):
        for v in (0.0, float(w) - 1.0, float(w), float(np.float32(w))):
            f = np.float32(v)
            extra += [f, np.nextafter(f, np.float32(np.inf)), np.nextafter(f, np.float32(-np.inf))]
    g = np.concatenate([g, np.array(extra, np.float32),
                        np.array([-0.0, 0.0, np.inf, -np.inf, 2.0 ** 31, -2.0 ** 31], np.float32)])
    g = g[~np.isnan(g)]
    fl = _f2i_rd(g)
    for w in (1, 7, 1100, 2 ** 24 - 1, 2 ** 24, 2 ** 24 + 1, 2 ** 24 + 3, 2 ** 31 - 1):
        fw = np.float32(w)
        ref = (np.float32(0.0) <= g) & (g < fw)
        bound = min(w, int(fw))
        got = (fl >= 0) & (fl < bound)   # the unsigned compare of an int32
        assert np.array_equal(ref, got), w
        inside = g[ref].astype(np.float64)
        assert np.array_equal(np.trunc(inside), np.floor(inside))
        assert np.all(fl[ref] < w)   # the cell read stays inside the map


def test_bresenham_walk_that_skips_its_end(oracle_mod):
    """A start whose fraction is 1 - ulp rounds up where the walk crosses a power of two
    (999.99994 + 24 -> 1025.0) and skips its end cell 1024; the reference's loop never ends there.
    The oracle's loop bound returns max_range after |x1 - x0| + 4 steps."""
    occ = np.zeros((64, 1100), np.uint8)
    m = oracle_mod.OracleMethod(occ, "bl", 23.5)
    y = float(np.float32(1000.0) - np.float32(2.0 ** -14))
    r, steps = m.calc_range_steps(5.5, y, math.pi / 2)
    assert r == np.float32(23.5) and steps == 28
    r2, steps2 = m.calc_range_steps(5.5, 999.5, math.pi / 2)   # a neighbour that meets its end
    assert r2 == np.float32(23.5) and steps2 <= 26
