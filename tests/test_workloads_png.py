"""Seeded workload generators and the PNG map loader (host-only)."""
import os
import struct
import zlib

import numpy as np
import pytest

from range_libc_gb300 import workloads as W
from range_libc_gb300.range_libc import png_occupancy


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


def _filter_rows(rows, bpp, filters):
    """Scanlines with PNG filter bytes: filters[y] in 0..4 applied to row y."""
    out = b""
    prev = np.zeros(len(rows[0]), np.int32)
    for r, ft in zip(rows, filters):
        cur = np.frombuffer(r, np.uint8).astype(np.int32)
        a = np.concatenate([np.zeros(bpp, np.int32), cur[:-bpp]])
        c = np.concatenate([np.zeros(bpp, np.int32), prev[:-bpp]])
        b = prev
        if ft == 0:
            pred = np.zeros_like(cur)
        elif ft == 1:
            pred = a
        elif ft == 2:
            pred = b
        elif ft == 3:
            pred = (a + b) >> 1
        else:
            p = a + b - c
            pa, pb, pc = np.abs(p - a), np.abs(p - b), np.abs(p - c)
            pred = np.where((pa <= pb) & (pa <= pc), a, np.where(pb <= pc, b, c))
        out += bytes([ft]) + ((cur - pred) & 255).astype(np.uint8).tobytes()
        prev = cur
    return out


def _png(path, samples, color_type, bit_depth=8, filters=None, palette=None, level=6, strategy=None,
         idat_parts=1, interlace=0, corrupt=None):
    """Write samples [h, w, channels] (integers < 2**bit_depth) as a PNG."""
    h, w, ch = samples.shape
    rows = []
    for y in range(h):
        if bit_depth < 8:
            bits = np.unpackbits(samples[y, :, 0].astype(np.uint8)[:, None], axis=1)[:, 8 - bit_depth:]
            rows.append(np.packbits(bits.ravel()).tobytes())
        elif bit_depth == 16:
            rows.append(samples[y].astype(">u2").tobytes())
        else:
            rows.append(samples[y].astype(np.uint8).tobytes())
    bpp = max(1, ch * bit_depth // 8)
    raw = _filter_rows(rows, bpp, filters if filters is not None else [0] * h)
    if strategy is None:
        z = zlib.compress(raw, level)
    else:
        co = zlib.compressobj(level, zlib.DEFLATED, 15, 9, strategy)
        z = co.compress(raw) + co.flush()
    if corrupt == "adler":
        z = z[:-1] + bytes([z[-1] ^ 1])

    def chunk(t, b):
        crc = zlib.crc32(t + b) & 0xFFFFFFFF
        if corrupt == "crc" and t == b"IDAT":
            crc ^= 1
        return struct.pack(">I", len(b)) + t + b + struct.pack(">I", crc)

    body = chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, bit_depth, color_type, 0, 0, interlace))
    if palette is not None:
        body += chunk(b"PLTE", palette.astype(np.uint8).tobytes())
    body += chunk(b"tEXt", b"Comment\x00ancillary chunks are skipped")
    cuts = np.linspace(0, len(z), idat_parts + 1).astype(int)
    for i in range(idat_parts):
        body += chunk(b"IDAT", z[cuts[i]:cuts[i + 1]])
    data = b"\x89PNG\r\n\x1a\n" + body + chunk(b"IEND", b"")
    if corrupt == "truncate":
        data = data[: len(data) // 2]
    with open(path, "wb") as f:
        f.write(data)


def _expected(rgb, threshold=128.0):
    """grid[x][y] of the reference's loader for 8-bit RGB pixels [h, w, 3]."""
    r, g, b = (rgb[..., k].astype(np.float32).astype(np.float64) for k in (2, 1, 0))
    gray = (0.229 * r + 0.587 * g + 0.114 * b).astype(np.float32).astype(np.int32)
    return np.ascontiguousarray((gray.astype(np.float32) < np.float32(threshold)).T, dtype=np.uint8)


CASES = [   # (colour type, bit depth)
    (0, 1), (0, 2), (0, 4), (0, 8), (0, 16), (2, 8), (2, 16), (3, 1), (3, 2), (3, 4), (3, 8),
    (4, 8), (4, 16), (6, 8), (6, 16),
]


@pytest.mark.parametrize("ct,bd", CASES)
def test_png_decoder_formats(tmp_path, ct, bd):
    """Every colour type and bit depth, all five filters, stored / fixed / dynamic deflate blocks and
    split IDAT chunks, against the reference loader's rule computed from the pixels."""
    rng = np.random.default_rng(ct * 100 + bd)
    h, w = 23, 37
    ch = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ct]
    top = (1 << bd) - 1
    pal = None
    if ct == 3:
        pal = rng.integers(0, 256, (top + 1, 3))
        samples = rng.integers(0, top + 1, (h, w, 1))
        rgb = pal[samples[..., 0]]
    else:
        samples = rng.integers(0, top + 1, (h, w, ch))
        eight = samples >> 8 if bd == 16 else (samples * 255 // top if bd < 8 else samples)
        rgb = np.repeat(eight[..., :1], 3, axis=2) if ct in (0, 4) else eight[..., :3]
    for k, (level, strategy, parts) in enumerate(((0, None, 1), (9, zlib.Z_FIXED, 3), (6, None, 2), (1, zlib.Z_RLE, 1))):
        f = tmp_path / f"m{k}.png"
        _png(f, samples, ct, bd, filters=[(y + k) % 5 for y in range(h)], palette=pal, level=level,
             strategy=strategy, idat_parts=parts)
        for thr in (128.0, 37.5, 255.0):
            assert np.array_equal(png_occupancy(str(f), thr), _expected(rgb, thr)), (k, thr)


def test_png_occupancy_threshold_and_orientation(tmp_path):
    img = np.full((3, 5, 1), 255, np.uint8)   # rows x cols
    img[1, 4] = 0                             # row 1, col 4 is dark
    _png(tmp_path / "m.png", img, 0)
    occ = png_occupancy(str(tmp_path / "m.png"), 128.0)
    assert occ.shape == (5, 3)                # grid[x][y]: x = column, y = row
    assert occ[4, 1] == 1 and occ.sum() == 1


@pytest.mark.parametrize("bad", ["crc", "adler", "truncate", "interlaced", "palette", "missing", "not_png"])
def test_png_decoder_rejects(tmp_path, bad):
    from range_libc_gb300._lib import RLC_ERR_IO, RangeLibError
    f = tmp_path / "bad.png"
    px = np.full((4, 4, 1), 200, np.uint8)
    if bad in ("crc", "adler", "truncate"):
        _png(f, px, 0, corrupt=bad)
    elif bad == "interlaced":
        _png(f, px, 0, interlace=1)
    elif bad == "palette":
        _png(f, np.full((4, 4, 1), 3, np.uint8), 3, palette=np.zeros((2, 3), np.uint8))
    elif bad == "not_png":
        f.write_bytes(b"GIF89a" + bytes(40))
    with pytest.raises(RangeLibError) as e:
        png_occupancy(str(f))
    assert e.value.code == RLC_ERR_IO


def test_png_save_round_trip(tmp_path):
    """OMap::save writes 8-bit grey (occupied black); the decoder reads the same grid back."""
    from range_libc_gb300 import _lib
    occ = W.rect_disk_map(300, 5)[:300, :217].copy()
    f = str(tmp_path / "s.png")
    assert _lib.lib().rlc_png_save_occupancy(f.encode(), occ.ctypes.data, occ.shape[0], occ.shape[1]) == 0
    assert np.array_equal(png_occupancy(f), occ)
    assert open(f, "rb").read(8) == b"\x89PNG\r\n\x1a\n"
    with open(f, "rb") as fh:   # a standard zlib stream: Python's zlib inflates it
        data = fh.read()
    pos, idat = 8, b""
    while pos < len(data):
        ln, typ = struct.unpack(">I4s", data[pos:pos + 8])
        if typ == b"IDAT":
            idat += data[pos + 8:pos + 8 + ln]
        pos += 12 + ln
    raw = np.frombuffer(zlib.decompress(idat), np.uint8).reshape(217, 301)
    assert (raw[:, 0] == 0).all() and np.array_equal(raw[:, 1:] == 0, occ.T == 1)


def test_png_occupancy_matches_reference_loader():
    """The reference's own small fixture maps, loaded by the reference (golden) and by us."""
    import oracle as O
    ref_maps = os.path.join(O.REF_SRC, "maps")
    gold = np.load(os.path.join(os.path.dirname(__file__), "golden", "reference_vectors.npz"))
    if not os.path.isdir(ref_maps):
        pytest.skip("reference maps not present")
    for f, name in (("single_pixel.map.png", "single_pixel"), ("quad.map.png", "quad"), ("small.map.png", "small")):
        assert np.array_equal(png_occupancy(os.path.join(ref_maps, f), 128.0), gold[f"{name}/occ"])


def test_cpp_omap_png_constructor_and_save(tmp_path):
    """ranges::OMap(filename, threshold) and OMap::save from C++ (include/RangeLib.h), host only."""
    import subprocess
    from range_libc_gb300 import _lib
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    lib = _lib.library_path()
    exe = tmp_path / "png_caller"
    subprocess.check_call(["g++", "-std=c++14", "-O2", "-I", os.path.join(root, "include"),
                           os.path.join(root, "tests", "cpp", "png_caller.cpp"), "-o", str(exe),
                           "-L", os.path.dirname(lib), "-lrangelibc_gb300", f"-Wl,-rpath,{os.path.dirname(lib)}"])
    rng = np.random.default_rng(3)
    rgb = rng.integers(0, 256, (19, 31, 3))
    _png(tmp_path / "c.png", rgb, 2, filters=[y % 5 for y in range(19)])
    for thr in ("128", "90.5"):
        subprocess.check_call([str(exe), str(tmp_path / "c.png"), thr, str(tmp_path / "o.bin"), str(tmp_path / "s.png")])
        buf = (tmp_path / "o.bin").read_bytes()
        w, h, err = np.frombuffer(buf[:12], np.int32)
        assert (w, h, err) == (31, 19, 0)
        assert np.array_equal(np.frombuffer(buf[12:], np.uint8).reshape(w, h), _expected(rgb, float(thr)))
    r = subprocess.run([str(exe), str(tmp_path / "none.png"), "128", str(tmp_path / "o.bin"), str(tmp_path / "s.png")],
                       capture_output=True, text=True)
    assert r.returncode == 0 and "ERROR" in r.stdout
    assert tuple(np.frombuffer((tmp_path / "o.bin").read_bytes()[:12], np.int32)) == (0, 0, 1)


def test_png_decoder_survives_corrupt_files(tmp_path):
    """Mutated PNGs -- flipped bits in the deflate stream, scanlines with arbitrary filter bytes and
    lengths recompressed into valid streams, damaged headers -- decode or raise RangeLibError, never
    read out of bounds (the same corpus, 4,000 files, ran clean under AddressSanitizer and
    UndefinedBehaviorSanitizer)."""
    import random
    from range_libc_gb300._lib import RangeLibError
    rnd = random.Random(11)
    rng = np.random.default_rng(5)
    bases = []
    for k, (ct, bd, ch) in enumerate(((0, 8, 1), (2, 8, 3), (6, 16, 4), (3, 4, 1), (0, 1, 1))):
        top = (1 << bd) - 1
        pal = rng.integers(0, 256, (top + 1, 3)) if ct == 3 else None
        f = tmp_path / f"base{k}.png"
        _png(f, rng.integers(0, top + 1, (9, 13, ch)), ct, bd, filters=[y % 5 for y in range(9)], palette=pal)
        bases.append(f.read_bytes())

    def chunks(b):
        pos, res = 8, []
        while pos + 12 <= len(b):
            ln = struct.unpack(">I", b[pos:pos + 4])[0]
            res.append((b[pos + 4:pos + 8], b[pos + 8:pos + 8 + ln]))
            pos += 12 + ln
        return res

    decoded = 0
    for it in range(300):
        chs = chunks(rnd.choice(bases))
        idat = b"".join(d for t, d in chs if t == b"IDAT")
        mode = rnd.random()
        if mode < 0.4:
            z = bytearray(idat)
            for _ in range(rnd.randint(1, 6)):
                z[rnd.randrange(len(z))] ^= 1 << rnd.randrange(8)
            idat = bytes(z)
        elif mode < 0.7:
            raw = bytearray(zlib.decompress(idat))
            for _ in range(rnd.randint(1, 10)):
                raw[rnd.randrange(len(raw))] = rnd.randrange(256)
            if rnd.random() < 0.3:
                raw = raw[:rnd.randrange(len(raw))]
            idat = zlib.compress(bytes(raw))
        else:
            ih = bytearray(chs[0][1])
            ih[rnd.randrange(13)] = rnd.randrange(256)
            chs[0] = (b"IHDR", bytes(ih))
        body = [(t, d) for t, d in chs if t not in (b"IDAT", b"IEND")] + [(b"IDAT", idat), (b"IEND", b"")]
        data = b"\x89PNG\r\n\x1a\n" + b"".join(struct.pack(">I", len(d)) + t + d +
                                                struct.pack(">I", zlib.crc32(t + d) & 0xFFFFFFFF) for t, d in body)
        f = tmp_path / "m.png"
        f.write_bytes(data)
        try:
            occ = png_occupancy(str(f))
            assert occ.ndim == 2 and occ.dtype == np.uint8
            decoded += 1
        except RangeLibError:
            pass
    assert 0 < decoded < 300
