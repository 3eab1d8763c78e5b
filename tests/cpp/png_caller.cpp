// A C++ caller of ranges::OMap's PNG constructor and save (include/RangeLib.h); host code only.
//
// usage: png_caller <in.png> <threshold> <out.bin> <saved.png>
//   out.bin: int32 width, height, has_error; uint8 grid[x][y] at x * height + y
//   saved.png: the map written back by OMap::save
#include "RangeLib.h"

#include <cstdio>
#include <cstdlib>

int main(int argc, char** argv) {
    if (argc != 5) return 2;
    ranges::OMap m(argv[1], (float)std::atof(argv[2]));
    FILE* o = std::fopen(argv[3], "wb");
    if (!o) return 2;
    const int hdr[3] = {(int)m.width, (int)m.height, m.error() ? 1 : 0};
    std::fwrite(hdr, sizeof(int), 3, o);
    const std::vector<uint8_t> occ = m.occupancy();
    std::fwrite(occ.data(), 1, occ.size(), o);
    std::fclose(o);
    if (m.error()) return 0;
    if (m.save(argv[4])) return 3;
    ranges::OMap back(argv[4]);
    if (back.error() || back.grid != m.grid || back.fn != argv[4]) return 4;
    return 0;
}
