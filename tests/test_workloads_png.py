"""Seeded workload generators and the PNG map loader (host-only)."""
import os
import struct
import zlib

import numpy as np
import pytest

from range_libc_gb300 import workloads as W
from range_libc_gb300.range_libc import _read_png_rgba, png_occupancy


def test_rect_disk_map_is_seeded_and_bordered():
    a, b = W.rect_disk_map(512, 1000), W.rect_disk_map(512, 1000)
    assert np.array_equal(a, b)
    assert a[0].all() and a[-1].all() and a[:, 0].all() and a[:, -1].all()
    assert 0.12 < a.mean() < 0.25
    big = W.rect_disk_map(2048, 3000)
    assert 0.12 < big.mean() < 0.25


def test_corridor_map_structure():
    occ = W.corridor_map(2048, 2000)
    assert occ.shape == (2048, 2048) and 0.02 < occ.mean() < 0.1
    assert np.array_equal(occ, W.corridor_map(2048, 2000))


def test_free_cell_queries_land_on_free_cells():
    occ = W.rect_disk_map(256, 3)
    q = W.free_cell_queries(occ, 5000, 4)
    assert q.dtype == np.float32 and q.shape == (5000, 3)
    assert not occ[q[:, 0].astype(int), q[:, 1].astype(int)].any()
    assert (q[:, 2] >= 0).all() and (q[:, 2] < 2 * np.pi + 1e-6).all()


def test_sensor_table_columns_normalised():
    t = W.sensor_table(201)
    assert t.shape == (201, 201) and t.dtype == np.float64
    assert np.allclose(t.sum(axis=0), 1.0)


def test_particle_filter_step_shapes():
    wl = W.particle_filter_step()
    assert wl.ins.shape == (4000, 3) and wl.angles.shape == (61,) and wl.obs.shape == (61,)
    assert wl.table.shape == (201, 201) and wl.occ.shape == (2048, 2048)
    assert np.isclose(wl.angles[0], -0.75 * np.pi) and np.isclose(wl.angles[-1], 0.75 * np.pi)


def test_uneven_batch_specs_ranges():
    specs = W.uneven_batch_specs()
    assert len(specs) == 32
    for s in specs:
        assert s.side in (512, 1024, 2048, 4096)
        assert 500 <= s.n_particles <= 20000 and 30 <= s.n_beams <= 1081 and 100 <= s.max_range <= 400


def _png(path, pixels, color_type, bit_depth=8, filt=0):
    h, w = pixels.shape[:2]
    rows = []
    if bit_depth < 8:
        for y in range(h):
            bits = np.unpackbits(pixels[y].astype(np.uint8)[:, None], axis=1)[:, 8 - bit_depth:]
            rows.append(np.packbits(bits.ravel()).tobytes())
    else:
        rows = [pixels[y].tobytes() for y in range(h)]
    raw = b""
    prev = b"\x00" * len(rows[0])
    for r in rows:
        if filt == 2:   # Up
            r2 = bytes((a - b) & 255 for a, b in zip(r, prev))
            raw += b"\x02" + r2
        else:
            raw += b"\x00" + r
        prev = r

    def chunk(t, b):
        return struct.pack(">I", len(b)) + t + b + struct.pack(">I", zlib.crc32(t + b) & 0xFFFFFFFF)

    with open(path, "wb") as f:
        f.write(b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, bit_depth, color_type, 0, 0, 0))
                + chunk(b"IDAT", zlib.compress(raw)) + chunk(b"IEND", b""))


def test_png_decoder_colour_types(tmp_path):
    rng = np.random.default_rng(0)
    g = rng.integers(0, 256, (7, 5), dtype=np.uint8)
    _png(tmp_path / "g.png", g, 0)
    assert np.array_equal(_read_png_rgba(str(tmp_path / "g.png"))[..., 0], g)
    rgb = rng.integers(0, 256, (4, 6, 3), dtype=np.uint8)
    _png(tmp_path / "rgb.png", rgb, 2, filt=2)
    assert np.array_equal(_read_png_rgba(str(tmp_path / "rgb.png"))[..., :3], rgb)
    rgba = rng.integers(0, 256, (3, 3, 4), dtype=np.uint8)
    _png(tmp_path / "rgba.png", rgba, 6)
    assert np.array_equal(_read_png_rgba(str(tmp_path / "rgba.png")), rgba)
    b1 = rng.integers(0, 2, (5, 6), dtype=np.uint8)
    _png(tmp_path / "b1.png", b1, 0, bit_depth=1)
    assert np.array_equal(_read_png_rgba(str(tmp_path / "b1.png"))[..., 0], b1 * 255)


def test_png_occupancy_threshold_and_orientation(tmp_path):
    img = np.full((3, 5), 255, np.uint8)    # rows x cols
    img[1, 4] = 0                           # row 1, col 4 is dark
    _png(tmp_path / "m.png", img, 0)
    occ = png_occupancy(str(tmp_path / "m.png"), 128.0)
    assert occ.shape == (5, 3)              # grid[x][y]: x = column, y = row
    assert occ[4, 1] == 1 and occ.sum() == 1


def test_png_occupancy_matches_reference_loader():
    """The reference's own small fixture maps, loaded by the reference (golden) and by us."""
    ref_maps = os.path.join(os.environ.get("RLC_REFERENCE_DIR", "/root/reference"), "maps")
    gold = np.load(os.path.join(os.path.dirname(__file__), "golden", "reference_vectors.npz"))
    if not os.path.isdir(ref_maps):
        pytest.skip("reference maps not present")
    for f, name in (("single_pixel.map.png", "single_pixel"), ("quad.map.png", "quad"), ("small.map.png", "small")):
        assert np.array_equal(png_occupancy(os.path.join(ref_maps, f), 128.0), gold[f"{name}/occ"])
