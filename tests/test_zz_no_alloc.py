"""rlc_distance_transform_noalloc: the distance transform without device allocation.

Callers that may not call cudaMalloc (real-time loops that forbid allocation
after start-up, hosts whose device memory belongs to another allocator) get
one entry point whose scratch is a fixed device array inside the library.
This file checks it through the C ABI against the ordinary entry point
(rlc_map_distance_transform), bit for bit, on two calls in a row that reuse
the same scratch, and checks that oversized maps are refused.  It is named so
that pytest collects it last.
"""
import ctypes as C

import numpy as np
import pytest

from range_libc_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _reference_dt(rl, occ):
    """Distance transform through the existing entry point (map handle, allocating)."""
    h = C.c_void_p()
    o = np.ascontiguousarray(occ, np.uint8)
    rl._lib.call("rlc_map_create", o.ctypes.data_as(rl._lib._u8p), o.shape[0], o.shape[1], C.byref(h))
    try:
        out = np.empty(o.shape, np.float32)
        rl._lib.call("rlc_map_distance_transform", h, out.ctypes.data_as(rl._lib._f32p))
    finally:
        rl._lib.lib().rlc_map_destroy(h)
    return out


def _noalloc_dt(rl, torch, occ):
    dev = torch.device("cuda:0")
    d_occ = torch.from_numpy(np.ascontiguousarray(occ, np.uint8)).to(dev)
    d_dt = torch.full(occ.shape, -1.0, dtype=torch.float32, device=dev)
    stream = C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    rl._lib.call("rlc_distance_transform_noalloc", C.c_void_p(d_occ.data_ptr()), occ.shape[0], occ.shape[1],
                 C.c_void_p(d_dt.data_ptr()), stream)
    torch.cuda.synchronize()
    return d_dt.cpu().numpy()


def test_noalloc_matches_allocating_entry_point(rl):
    torch = pytest.importorskip("torch")
    maps = [
        W.rect_disk_map(1024, 77),                                   # the largest allowed map
        np.ascontiguousarray(W.corridor_map(512, 78)[:300, :410]),   # smaller, non-square, after it
        np.ascontiguousarray(W.rect_disk_map(4096, 79)[:, :256]),    # the side limit with few rows
        np.ascontiguousarray(W.rect_disk_map(4096, 80)[:256, :]),    # and with few columns
    ]
    for occ in maps:   # two calls in a row share the scratch
        got = _noalloc_dt(rl, torch, occ)
        exp = _reference_dt(rl, occ)
        assert np.array_equal(got.view(np.uint32), exp.view(np.uint32))


def test_noalloc_rejects_oversized_maps(rl):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda:0")
    buf = torch.zeros(1025 * 1024, dtype=torch.uint8, device=dev)
    out = torch.zeros(1025 * 1024, dtype=torch.float32, device=dev)
    rc = rl._lib.lib().rlc_distance_transform_noalloc(C.c_void_p(buf.data_ptr()), 1025, 1024,
                                                      C.c_void_p(out.data_ptr()), None)
    assert rc == rl._lib.RLC_ERR_ARG
    assert b"exceeds the fixed scratch" in rl._lib.lib().rlc_last_error()
    rc = rl._lib.lib().rlc_distance_transform_noalloc(C.c_void_p(buf.data_ptr()), 5000, 10,
                                                      C.c_void_p(out.data_ptr()), None)
    assert rc == rl._lib.RLC_ERR_ARG


def test_noalloc_rejects_host_memory(rl):
    """Host buffers are refused before anything is launched (the kernels would read them as
    device addresses)."""
    torch = pytest.importorskip("torch")
    occ = np.zeros((16, 16), np.uint8)
    dt = np.zeros((16, 16), np.float32)
    dev = torch.device("cuda:0")
    d_occ = torch.zeros(256, dtype=torch.uint8, device=dev)
    d_dt = torch.zeros(256, dtype=torch.float32, device=dev)
    L = rl._lib.lib()
    for a, b in ((occ.ctypes.data, d_dt.data_ptr()), (d_occ.data_ptr(), dt.ctypes.data)):
        rc = L.rlc_distance_transform_noalloc(C.c_void_p(a), 16, 16, C.c_void_p(b), None)
        assert rc == rl._lib.RLC_ERR_ARG
        assert b"device memory of the current device" in L.rlc_last_error()
    torch.cuda.synchronize()
