"""Float-only forms of the reference's mixed float/double angle arithmetic, checked exhaustively.

discretize_theta (RangeLib.h:1287-1340) compares a float heading with the double constants
M_2PI and M_PI and subtracts M_PI in double.  The kernels use float-only forms (the FP64 pipe
of GB300 is slow); these tests show the forms are identical for every float they are used on.
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
