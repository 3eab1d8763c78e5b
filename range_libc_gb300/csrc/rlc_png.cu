// PNG map files for OMap(std::string, threshold) (RangeLib.h:159-201) and
// OMap::save (RangeLib.h:263-291): host code only.
//
// The decoder covers what the reference's maps use and more: colour types
// 0, 2, 3, 4, 6 at every bit depth PNG allows (16-bit samples keep their
// high byte, as the reference's decoder does when it delivers 8-bit RGBA),
// the five scanline filters, zlib streams with stored, fixed and dynamic
// Huffman blocks, and chunk CRC and Adler-32 checks.  Interlaced images are
// refused.  The encoder writes 8-bit grey with a run-length deflate stream.
#include "rangelibc.h"
#include "rlc_internal.cuh"

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace {

// ------------------------------------------------------------- checksums
struct CrcTable {
    uint32_t t[256];
    CrcTable() {
        for (uint32_t n = 0; n < 256; ++n) {
            uint32_t c = n;
            for (int k = 0; k < 8; ++k) c = (c & 1) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
            t[n] = c;
        }
    }
};

uint32_t crc32(const uint8_t* p, size_t n, uint32_t crc = 0) {
    static const CrcTable tab;
    uint32_t c = ~crc;
    for (size_t i = 0; i < n; ++i) c = tab.t[(c ^ p[i]) & 0xFF] ^ (c >> 8);
    return ~c;
}

uint32_t adler32(const uint8_t* p, size_t n) {
    uint32_t a = 1, b = 0;
    while (n) {
        const size_t k = n < 5552 ? n : 5552;   // largest run without overflow before the modulo
        for (size_t i = 0; i < k; ++i) {
            a += p[i];
            b += a;
        }
        a %= 65521u;
        b %= 65521u;
        p += k;
        n -= k;
    }
    return (b << 16) | a;
}

uint32_t be32(const uint8_t* p) { return (uint32_t)p[0] << 24 | (uint32_t)p[1] << 16 | (uint32_t)p[2] << 8 | p[3]; }

// ------------------------------------------------------------- inflate (RFC 1950 / 1951)
struct BitIn {
    const uint8_t* p;
    size_t n, pos = 0;
    uint64_t buf = 0;
    int cnt = 0;
    bool eof = false;
    BitIn(const uint8_t* d, size_t len) : p(d), n(len) {}
    unsigned get(int k) {   // k <= 16 bits, least significant first
        while (cnt < k) {
            if (pos >= n) {
                eof = true;
                return 0;
            }
            buf |= (uint64_t)p[pos++] << cnt;
            cnt += 8;
        }
        const unsigned v = (unsigned)(buf & ((1u << k) - 1));
        buf >>= k;
        cnt -= k;
        return v;
    }
    void to_byte() {
        buf >>= cnt & 7;
        cnt -= cnt & 7;
    }
};

// canonical Huffman code: count of codes per length and symbols in code order
struct Huffman {
    uint16_t count[16];
    uint16_t symbol[320];
};

// false when the lengths over-subscribe the code space
bool huffman_build(Huffman& h, const uint8_t* len, int n) {
    std::memset(h.count, 0, sizeof(h.count));
    for (int i = 0; i < n; ++i) h.count[len[i]]++;
    if (h.count[0] == n) return true;   // no codes (a block of literals only has no distances)
    int left = 1;
    for (int b = 1; b < 16; ++b) {
        left = (left << 1) - h.count[b];
        if (left < 0) return false;
    }
    uint16_t offs[16];
    offs[1] = 0;
    for (int b = 1; b < 15; ++b) offs[b + 1] = (uint16_t)(offs[b] + h.count[b]);
    for (int i = 0; i < n; ++i)
        if (len[i]) h.symbol[offs[len[i]]++] = (uint16_t)i;
    return true;
}

// next symbol, -1 on a code the table does not hold or at the end of the data
int huffman_decode(BitIn& in, const Huffman& h) {
    int code = 0, first = 0, index = 0;
    for (int b = 1; b < 16; ++b) {
        code |= (int)in.get(1);
        if (in.eof) return -1;
        const int c = h.count[b];
        if (code - first < c) return h.symbol[index + code - first];
        index += c;
        first = (first + c) << 1;
        code <<= 1;
    }
    return -1;
}

const uint16_t kLenBase[29] = {3, 4, 5, 6, 7, 8, 9, 10, 11, 13, 15, 17, 19, 23, 27, 31,
                               35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
const uint8_t kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const uint16_t kDistBase[30] = {1, 2, 3, 4, 5, 7, 9, 13, 17, 25, 33, 49, 65, 97, 129, 193,
                                257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
const uint8_t kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};

bool inflate_codes(BitIn& in, const Huffman& lit, const Huffman& dist, std::vector<uint8_t>& out, size_t cap,
                   std::string& why) {
    for (;;) {
        int sym = huffman_decode(in, lit);
        if (sym < 0) return why = "corrupt or truncated deflate data", false;
        if (sym < 256) {
            if (out.size() >= cap) return why = "more image data than the header allows", false;
            out.push_back((uint8_t)sym);
            continue;
        }
        if (sym == 256) return true;
        sym -= 257;
        if (sym >= 29) return why = "invalid deflate length code", false;
        const size_t len = kLenBase[sym] + in.get(kLenExtra[sym]);
        const int ds = huffman_decode(in, dist);
        if (ds < 0 || ds >= 30) return why = "invalid deflate distance code", false;
        const size_t d = kDistBase[ds] + in.get(kDistExtra[ds]);
        if (in.eof) return why = "truncated deflate data", false;
        if (d > out.size()) return why = "deflate distance before the start of the data", false;
        if (out.size() + len > cap) return why = "more image data than the header allows", false;
        const size_t from = out.size() - d;
        for (size_t i = 0; i < len; ++i) out.push_back(out[from + i]);
    }
}

bool inflate_zlib(const uint8_t* z, size_t n, size_t cap, std::vector<uint8_t>& out, std::string& why) {
    if (n < 6) return why = "zlib stream too short", false;
    if ((z[0] & 15) != 8 || (z[0] >> 4) > 7 || ((unsigned)z[0] << 8 | z[1]) % 31 != 0)
        return why = "bad zlib header", false;
    if (z[1] & 0x20) return why = "zlib preset dictionaries are not supported", false;
    BitIn in(z + 2, n - 2);
    out.clear();
    out.reserve(cap);
    static Huffman fixed_lit, fixed_dist;
    static const bool fixed_ready = [] {
        uint8_t l[288];
        for (int i = 0; i < 288; ++i) l[i] = i < 144 ? 8 : i < 256 ? 9 : i < 280 ? 7 : 8;
        huffman_build(fixed_lit, l, 288);
        for (int i = 0; i < 30; ++i) l[i] = 5;
        huffman_build(fixed_dist, l, 30);
        return true;
    }();
    (void)fixed_ready;
    int last = 0;
    do {
        last = (int)in.get(1);
        const unsigned type = in.get(2);
        if (in.eof) return why = "truncated deflate data", false;
        if (type == 0) {
            in.to_byte();
            const unsigned len = in.get(16), nlen = in.get(16);
            if (in.eof || (len ^ 0xFFFFu) != nlen) return why = "bad stored deflate block", false;
            if (out.size() + len > cap) return why = "more image data than the header allows", false;
            for (unsigned i = 0; i < len; ++i) out.push_back((uint8_t)in.get(8));
            if (in.eof) return why = "truncated deflate data", false;
        } else if (type == 1) {
            if (!inflate_codes(in, fixed_lit, fixed_dist, out, cap, why)) return false;
        } else if (type == 2) {
            const int nlit = (int)in.get(5) + 257, ndist = (int)in.get(5) + 1, ncode = (int)in.get(4) + 4;
            if (nlit > 286 || ndist > 30) return why = "bad dynamic deflate block", false;
            static const uint8_t order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
            uint8_t lens[320] = {0};
            for (int i = 0; i < ncode; ++i) lens[order[i]] = (uint8_t)in.get(3);
            Huffman lc;
            if (in.eof || !huffman_build(lc, lens, 19)) return why = "bad dynamic deflate block", false;
            int i = 0;
            while (i < nlit + ndist) {
                const int sym = huffman_decode(in, lc);
                if (sym < 0) return why = "bad dynamic deflate block", false;
                if (sym < 16) {
                    lens[i++] = (uint8_t)sym;
                    continue;
                }
                int rep = 0;
                uint8_t v = 0;
                if (sym == 16) {
                    if (i == 0) return why = "bad dynamic deflate block", false;
                    v = lens[i - 1];
                    rep = 3 + (int)in.get(2);
                } else if (sym == 17) {
                    rep = 3 + (int)in.get(3);
                } else {
                    rep = 11 + (int)in.get(7);
                }
                if (in.eof || i + rep > nlit + ndist) return why = "bad dynamic deflate block", false;
                while (rep--) lens[i++] = v;
            }
            if (lens[256] == 0) return why = "deflate block without an end code", false;
            Huffman lit, dist;
            if (!huffman_build(lit, lens, nlit) || !huffman_build(dist, lens + nlit, ndist))
                return why = "bad dynamic deflate block", false;
            if (!inflate_codes(in, lit, dist, out, cap, why)) return false;
        } else {
            return why = "invalid deflate block type", false;
        }
    } while (!last);
    in.to_byte();
    uint8_t a[4];
    for (int k = 0; k < 4; ++k) a[k] = (uint8_t)in.get(8);
    if (in.eof) return why = "zlib stream without its Adler-32", false;
    if (be32(a) != adler32(out.data(), out.size())) return why = "zlib Adler-32 mismatch", false;
    return true;
}

// ------------------------------------------------------------- PNG decoding
struct Png {
    uint32_t w = 0, h = 0;
    int depth = 0, color = 0, interlace = 0;
    std::vector<uint8_t> palette;   // RGB triples
    std::vector<uint8_t> idat;
};

int channels_of(int color) { return color == 0 || color == 3 ? 1 : color == 4 ? 2 : color == 2 ? 3 : 4; }

bool depth_allowed(int color, int depth) {
    switch (color) {
    case 0: return depth == 1 || depth == 2 || depth == 4 || depth == 8 || depth == 16;
    case 3: return depth == 1 || depth == 2 || depth == 4 || depth == 8;
    case 2: case 4: case 6: return depth == 8 || depth == 16;
    default: return false;
    }
}

// parses the chunks (all of them when `header_only` is false), checking every CRC
bool read_png(const char* path, bool header_only, Png& png, std::string& why) {
    FILE* f = std::fopen(path, "rb");
    if (!f) return why = std::string("cannot open ") + path, false;
    std::vector<uint8_t> file;
    uint8_t buf[65536];
    size_t got;
    while ((got = std::fread(buf, 1, sizeof(buf), f)) > 0) file.insert(file.end(), buf, buf + got);
    std::fclose(f);
    static const uint8_t sig[8] = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1A, '\n'};
    if (file.size() < 8 || std::memcmp(file.data(), sig, 8) != 0) return why = "not a PNG file", false;
    size_t pos = 8;
    bool have_header = false, have_end = false;
    while (pos + 12 <= file.size()) {
        const uint32_t len = be32(&file[pos]);
        if (len > file.size() - pos - 12) return why = "truncated PNG chunk", false;
        const uint8_t* type = &file[pos + 4];
        const uint8_t* data = type + 4;
        if (crc32(type, len + 4) != be32(data + len)) return why = "PNG chunk CRC mismatch", false;
        if (!have_header && std::memcmp(type, "IHDR", 4) != 0) return why = "PNG does not start with IHDR", false;
        if (std::memcmp(type, "IHDR", 4) == 0) {
            if (len != 13) return why = "bad IHDR", false;
            png.w = be32(data);
            png.h = be32(data + 4);
            png.depth = data[8];
            png.color = data[9];
            png.interlace = data[12];
            if (png.w == 0 || png.h == 0 || png.w > 0x7FFFFFFFu || png.h > 0x7FFFFFFFu)
                return why = "bad PNG image size", false;
            if (!depth_allowed(png.color, png.depth)) return why = "bad PNG colour type / bit depth", false;
            if (data[10] != 0 || data[11] != 0 || png.interlace > 1) return why = "bad PNG compression or filter method", false;
            have_header = true;
            if (header_only) return true;
        } else if (std::memcmp(type, "PLTE", 4) == 0) {
            if (len % 3 || len > 768) return why = "bad PLTE", false;
            png.palette.assign(data, data + len);
        } else if (std::memcmp(type, "IDAT", 4) == 0) {
            png.idat.insert(png.idat.end(), data, data + len);
        } else if (std::memcmp(type, "IEND", 4) == 0) {
            have_end = true;
            break;
        } else if (!(type[0] & 0x20)) {
            return why = "unknown critical PNG chunk", false;
        }
        pos += 12 + (size_t)len;
    }
    if (!have_header) return why = "PNG without IHDR", false;
    if (!have_end) return why = "PNG without IEND", false;
    return true;
}

int paeth(int a, int b, int c) {
    const int p = a + b - c, pa = p > a ? p - a : a - p, pb = p > b ? p - b : b - p, pc = p > c ? p - c : c - p;
    return (pa <= pb && pa <= pc) ? a : (pb <= pc ? b : c);
}

// pixel(x, y, rgb) for every pixel, with its 8-bit RGB
template <class F>
bool decode_pixels(Png& png, F pixel, std::string& why) {
    if (png.interlace) return why = "interlaced PNGs are not supported", false;
    if (png.color == 3 && png.palette.empty()) return why = "palette image without PLTE", false;
    const int ch = channels_of(png.color);
    const size_t bits = (size_t)png.w * ch * png.depth;
    const size_t stride = (bits + 7) / 8, bpp = std::max<size_t>(1, (size_t)ch * png.depth / 8);
    const double raw_bytes = (double)png.h * (double)(stride + 1);
    if (raw_bytes > 8e9) return why = "PNG image too large", false;
    std::vector<uint8_t> raw;
    if (!inflate_zlib(png.idat.data(), png.idat.size(), (size_t)raw_bytes, raw, why)) return false;
    if (raw.size() != (size_t)raw_bytes) return why = "PNG image data shorter than the header says", false;
    std::vector<uint8_t>().swap(png.idat);
    // undo the scanline filters in place; row y's bytes follow its filter byte
    for (size_t y = 0; y < png.h; ++y) {
        uint8_t* row = &raw[y * (stride + 1)];
        const int ft = row[0];
        uint8_t* cur = row + 1;
        const uint8_t* prev = y ? &raw[(y - 1) * (stride + 1) + 1] : nullptr;
        if (ft > 4) return why = "bad PNG filter type", false;
        for (size_t i = 0; i < stride; ++i) {
            const int a = i >= bpp ? cur[i - bpp] : 0, b = prev ? prev[i] : 0;
            const int c = (prev && i >= bpp) ? prev[i - bpp] : 0;
            int pred = 0;
            switch (ft) {
            case 1: pred = a; break;
            case 2: pred = b; break;
            case 3: pred = (a + b) >> 1; break;
            case 4: pred = paeth(a, b, c); break;
            default: break;
            }
            cur[i] = (uint8_t)(cur[i] + pred);
        }
    }
    const int maxv = (1 << png.depth) - 1;
    const size_t ncolors = png.palette.size() / 3;
    uint8_t o[3];
    for (size_t y = 0; y < png.h; ++y) {
        const uint8_t* row = &raw[y * (stride + 1) + 1];
        for (size_t x = 0; x < png.w; ++x) {
            if (png.depth < 8) {   // grey or palette index packed most significant bits first
                const size_t bit = x * png.depth;
                const int v = (row[bit >> 3] >> (8 - png.depth - (int)(bit & 7))) & maxv;
                if (png.color == 3) {
                    if ((size_t)v >= ncolors) return why = "PNG palette index out of range", false;
                    std::memcpy(o, &png.palette[3 * (size_t)v], 3);
                } else {
                    o[0] = o[1] = o[2] = (uint8_t)(v * 255 / maxv);
                }
            } else {
                const size_t step = png.depth / 8;   // bytes per sample; 16-bit samples keep the high byte
                const uint8_t* px = row + x * ch * step;
                switch (png.color) {
                case 0: case 4: o[0] = o[1] = o[2] = px[0]; break;
                case 3:
                    if (px[0] >= ncolors) return why = "PNG palette index out of range", false;
                    std::memcpy(o, &png.palette[3 * (size_t)px[0]], 3);
                    break;
                default: o[0] = px[0]; o[1] = px[step]; o[2] = px[2 * step]; break;
                }
            }
            pixel(x, y, o);
        }
    }
    return true;
}

// ------------------------------------------------------------- PNG encoding
struct BitOut {
    std::vector<uint8_t>& out;
    uint32_t buf = 0;
    int cnt = 0;
    explicit BitOut(std::vector<uint8_t>& o) : out(o) {}
    void put(uint32_t v, int k) {   // least significant bit first
        buf |= v << cnt;
        cnt += k;
        while (cnt >= 8) {
            out.push_back((uint8_t)buf);
            buf >>= 8;
            cnt -= 8;
        }
    }
    void huff(uint32_t code, int k) {   // Huffman codes go most significant bit first
        uint32_t r = 0;
        for (int i = 0; i < k; ++i) r |= ((code >> i) & 1u) << (k - 1 - i);
        put(r, k);
    }
    void flush() {
        if (cnt) out.push_back((uint8_t)buf);
        buf = 0;
        cnt = 0;
    }
};

void fixed_literal(BitOut& b, int v) {
    if (v < 144) b.huff(0x30 + v, 8);
    else if (v < 256) b.huff(0x190 + v - 144, 9);
    else if (v < 280) b.huff(v - 256, 7);
    else b.huff(0xC0 + v - 280, 8);
}

// one fixed-Huffman block: literals, and runs of the previous byte as distance-1 matches
void deflate_runs(const std::vector<uint8_t>& raw, std::vector<uint8_t>& z) {
    z.push_back(0x78);
    z.push_back(0x01);
    BitOut b(z);
    b.put(1, 1);   // last block
    b.put(1, 2);   // fixed Huffman codes
    size_t i = 0;
    while (i < raw.size()) {
        size_t run = 0;
        if (i > 0)
            while (i + run < raw.size() && run < 258 && raw[i + run] == raw[i - 1]) ++run;
        if (run >= 3) {
            int s = 28;
            while (kLenBase[s] > run) --s;
            fixed_literal(b, 257 + s);
            b.put((uint32_t)(run - kLenBase[s]), kLenExtra[s]);
            b.huff(0, 5);   // distance code 0: distance 1
            i += run;
        } else {
            fixed_literal(b, raw[i]);
            ++i;
        }
    }
    fixed_literal(b, 256);
    b.flush();
    const uint32_t ad = adler32(raw.data(), raw.size());
    for (int k = 3; k >= 0; --k) z.push_back((uint8_t)(ad >> (8 * k)));
}

void put_chunk(std::vector<uint8_t>& f, const char* type, const std::vector<uint8_t>& data) {
    const uint32_t n = (uint32_t)data.size();
    for (int k = 3; k >= 0; --k) f.push_back((uint8_t)(n >> (8 * k)));
    const size_t at = f.size();
    f.insert(f.end(), type, type + 4);
    f.insert(f.end(), data.begin(), data.end());
    const uint32_t c = crc32(&f[at], 4 + data.size());
    for (int k = 3; k >= 0; --k) f.push_back((uint8_t)(c >> (8 * k)));
}

}  // namespace

int rlc_png_occupancy(const char* path, float threshold, uint8_t* occ, int* width, int* height) {
    if (!path || !width || !height) return rlc::set_last_error(RLC_ERR_ARG, "null argument");
    Png png;
    std::string why;
    if (!read_png(path, occ == nullptr, png, why)) return rlc::set_last_error(RLC_ERR_IO, why.c_str());
    if ((uint64_t)png.w * png.h > 0x7FFFFFFFull) return rlc::set_last_error(RLC_ERR_IO, "PNG image too large");
    if (!occ) {
        *width = (int)png.w;
        *height = (int)png.h;
        return RLC_OK;
    }
    if (*width != (int)png.w || *height != (int)png.h)
        return rlc::set_last_error(RLC_ERR_ARG, "width / height differ from the file's (read them first)");
    const size_t H = png.h;
    auto pixel = [&](size_t x, size_t y, const uint8_t* p) {
        // the reference takes r, g, b from bytes 2, 1, 0 of each RGBA pixel
        const float r = p[2], g = p[1], b = p[0];
        const float gray = (float)(0.229 * r + 0.587 * g + 0.114 * b);   // utils::rgb2gray
        occ[x * H + y] = (float)(int)gray < threshold ? 1 : 0;
    };
    if (!decode_pixels(png, pixel, why)) return rlc::set_last_error(RLC_ERR_IO, why.c_str());
    return RLC_OK;
}

int rlc_png_save_occupancy(const char* path, const uint8_t* occ, int width, int height) {
    if (!path || !occ) return rlc::set_last_error(RLC_ERR_ARG, "null argument");
    if (width <= 0 || height <= 0) return rlc::set_last_error(RLC_ERR_ARG, "width and height must be positive");
    const size_t W = (size_t)width, H = (size_t)height;
    std::vector<uint8_t> raw(H * (W + 1));
    for (size_t y = 0; y < H; ++y) {
        raw[y * (W + 1)] = 0;   // filter: none
        for (size_t x = 0; x < W; ++x) raw[y * (W + 1) + 1 + x] = occ[x * H + y] ? 0 : 255;
    }
    std::vector<uint8_t> z, f = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1A, '\n'};
    deflate_runs(raw, z);
    std::vector<uint8_t> ihdr(13, 0);
    for (int k = 0; k < 4; ++k) {
        ihdr[k] = (uint8_t)(W >> (24 - 8 * k));
        ihdr[4 + k] = (uint8_t)(H >> (24 - 8 * k));
    }
    ihdr[8] = 8;   // bit depth; colour type 0 (grey), deflate, adaptive filters, not interlaced
    put_chunk(f, "IHDR", ihdr);
    put_chunk(f, "IDAT", z);
    put_chunk(f, "IEND", {});
    FILE* out = std::fopen(path, "wb");
    if (!out) return rlc::set_last_error(RLC_ERR_IO, (std::string("cannot write ") + path).c_str());
    const bool ok = std::fwrite(f.data(), 1, f.size(), out) == f.size();
    if (std::fclose(out) != 0 || !ok) return rlc::set_last_error(RLC_ERR_IO, (std::string("cannot write ") + path).c_str());
    return RLC_OK;
}
