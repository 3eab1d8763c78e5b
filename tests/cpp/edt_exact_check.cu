// Host check of the distance transform's exact-comparison passes (rlc_map.cu: edt_col_exact,
// fh_line_exact, as launch_edt picks them for maps up to 16384 per side) against the oracle's
// Felzenszwalb-Huttenlocher transform, bit for bit.
//
//   edt_exact_check [--quick] [occupancy.u8 W H]...
//
// Each file holds W * H bytes (x-major, 1 = occupied).  Built-in cases: seeded random maps of
// many shapes and densities, sparse maps with full columns, maps whose pass 2 meets mostly
// FLT_MAX inputs, 4096 x 4096 maps whose squared distances approach 2 * 4095^2, and maps with a
// side above 4096 (up to 16384), whose sums f + q*q round in float.  Prints
// "<cases> cases, <n> mismatches" and exits non-zero on a mismatch.
#include "rlc_map.cu"

#include <cmath>
#include <cstring>
#include <random>
#include <vector>

extern "C" void orc_edt(const uint8_t* occ, int width, int height, float* dt_out);

namespace rlc {
int set_last_error(int code, const char*) { return code; }   // the map entry points are not called here
}

namespace {

struct HostIn {
    const float* g;
    size_t stride;
    float operator()(unsigned q) const { return g[q * stride]; }
};
struct HostOcc {   // pass 1 input: 0 on occupied cells, FLT_MAX elsewhere
    const uint8_t* occ;
    float operator()(unsigned q) const { return occ[q] ? 0.0f : FLT_MAX; }
};
struct HostOut {
    float* d;
    void operator()(unsigned q, float v) const { d[q] = v; }
};
struct HostSqrtOut {
    float* d;
    size_t stride;
    void operator()(unsigned q, float v) const { d[q * stride] = sqrtf(v); }
};

bool check(const std::vector<uint8_t>& occ, int W, int H, const char* what) {
    const int TY = (H + 7) >> 3, TX = (W + 7) >> 3;
    std::vector<uint64_t> bits((size_t)TX * TY, 0);
    for (int x = 0; x < W; ++x)
        for (int y = 0; y < H; ++y)
            if (occ[(size_t)x * H + y]) bits[(size_t)(x >> 3) * TY + (y >> 3)] |= 1ull << (((x & 7) << 3) | (y & 7));
    std::vector<float> g((size_t)W * H), dt((size_t)W * H), ref((size_t)W * H);
    std::vector<uint16_t> nx(TY + 1), sv(W > H ? W : H);
    std::vector<float> sf(W > H ? W : H);
    const bool closed_form = W <= rlc::kEdtExactSide && H <= rlc::kEdtExactSide;   // as launch_edt chooses
    for (int x = 0; x < W; ++x) {
        if (closed_form)
            rlc::edt_col_exact(bits.data() + (size_t)(x >> 3) * TY, (x & 7) << 3, H, TY, nx.data(), g.data() + (size_t)x * H);
        else
            rlc::fh_line_exact(HostOcc{occ.data() + (size_t)x * H}, HostOut{g.data() + (size_t)x * H}, (unsigned)H,
                               sv.data(), sf.data(), 1);
    }
    for (int y = 0; y < H; ++y)
        rlc::fh_line_exact(HostIn{g.data() + y, (size_t)H}, HostSqrtOut{dt.data() + y, (size_t)H}, (unsigned)W,
                           sv.data(), sf.data(), 1);
    orc_edt(occ.data(), W, H, ref.data());
    size_t bad = 0, first = 0;
    for (size_t i = 0; i < dt.size(); ++i)
        if (memcmp(&dt[i], &ref[i], sizeof(float)) != 0 && bad++ == 0) first = i;
    if (bad) printf("mismatch %s %dx%d: %zu cells, first %zu: %.9g vs %.9g\n", what, W, H, bad, first, dt[first], ref[first]);
    return bad == 0;
}

}  // namespace

int main(int argc, char** argv) {
    bool quick = false;
    int cases = 0, fails = 0;
    int a = 1;
    if (a < argc && strcmp(argv[a], "--quick") == 0) { quick = true; ++a; }
    for (; a + 2 < argc; a += 3) {
        const int W = atoi(argv[a + 1]), H = atoi(argv[a + 2]);
        if (W <= 0 || H <= 0 || W > rlc::kEdtIntSide || H > rlc::kEdtIntSide) { printf("bad size\n"); return 2; }
        std::vector<uint8_t> occ((size_t)W * H);
        FILE* f = fopen(argv[a], "rb");
        if (!f) { printf("cannot open %s\n", argv[a]); return 2; }
        const size_t r = fread(occ.data(), 1, occ.size(), f);
        fclose(f);
        if (r != occ.size()) { printf("short file %s\n", argv[a]); return 2; }
        ++cases;
        fails += !check(occ, W, H, argv[a]);
    }
    std::mt19937_64 rng(12345);
    const int sizes[][2] = {{1, 1}, {1, 7}, {7, 1}, {2, 2}, {3, 5}, {8, 8}, {9, 17}, {31, 33}, {64, 64}, {100, 37},
                            {37, 100}, {255, 257}, {513, 129}, {1024, 1024}, {4096, 3}, {3, 4096}, {2048, 2048}};
    const double dens[] = {0.0, 1.0, 0.0005, 0.01, 0.2, 0.5, 0.95};
    for (auto& s : sizes)
        for (double d : dens) {
            const int W = s[0], H = s[1];
            if ((size_t)W * H > 600000 && (quick || (d != 0.0005 && d != 0.2))) continue;
            std::vector<uint8_t> occ((size_t)W * H);
            std::bernoulli_distribution b(d);
            for (auto& o : occ) o = b(rng);
            ++cases;
            fails += !check(occ, W, H, "random");
        }
    for (int t = 0; t < 40; ++t) {   // a few obstacles, sometimes a full column
        const int W = 1 + (int)(rng() % 300), H = 1 + (int)(rng() % 300);
        std::vector<uint8_t> occ((size_t)W * H, 0);
        const int k = (int)(rng() % 4);
        for (int i = 0; i < k; ++i) occ[(rng() % W) * (size_t)H + rng() % H] = 1;
        if (t % 5 == 0)
            for (int y = 0; y < H; ++y) occ[(size_t)(rng() % W) * H + y] = 1;
        ++cases;
        fails += !check(occ, W, H, "sparse");
    }
    {   // the limit: a corner obstacle alone, then 50 scattered ones
        const int W = 4096, H = 4096;
        std::vector<uint8_t> occ((size_t)W * H, 0);
        occ[0] = 1;
        ++cases;
        fails += !check(occ, W, H, "corner4096");
        if (!quick) {
            std::fill(occ.begin(), occ.end(), 0);
            for (int i = 0; i < 50; ++i) occ[(rng() % W) * (size_t)H + rng() % H] = 1;
            ++cases;
            fails += !check(occ, W, H, "sparse4096");
        }
    }
    {   // pass 2 meets mostly FLT_MAX inputs: obstacles in a handful of columns or one row
        const int dims[][2] = {{4095, 4093}, {4096, 17}, {17, 4096}, {3001, 4096}};
        for (auto& dd : dims)
            for (int pat = 0; pat < 3; ++pat) {
                if (quick && (dd[0] > 2048 && dd[1] > 2048) && pat) continue;
                const int W = dd[0], H = dd[1];
                std::vector<uint8_t> occ((size_t)W * H, 0);
                if (pat == 0)
                    for (int c = 0; c < 3; ++c) {
                        const int x = (int)(rng() % W);
                        for (int i = 0; i < 5; ++i) occ[(size_t)x * H + rng() % H] = 1;
                    }
                if (pat == 1) {
                    const int y = (int)(rng() % H);
                    for (int x = 0; x < W; x += 1 + (int)(rng() % 700)) occ[(size_t)x * H + y] = 1;
                }
                if (pat == 2) {
                    occ[(size_t)(W - 1) * H + (H - 1)] = 1;
                    occ[(size_t)(W / 2) * H] = 1;
                }
                ++cases;
                fails += !check(occ, W, H, "flt_max_columns");
            }
    }
    {   // a side above 4096: both passes run the stack with integer comparisons (keys up to 2^29)
        const int dims[][2] = {{4097, 40}, {40, 4100}, {16384, 9}, {9, 16384}, {10976, 64}, {64, 10976}, {6000, 5000}};
        for (auto& dd : dims)
            for (int pat = 0; pat < 3; ++pat) {
                const int W = dd[0], H = dd[1];
                if (quick && (size_t)W * H > 1000000 && pat) continue;
                std::vector<uint8_t> occ((size_t)W * H, 0);
                if (pat == 0) {
                    std::bernoulli_distribution b(0.001);
                    for (auto& o : occ) o = b(rng);
                }
                if (pat == 1) occ[0] = 1;   // one corner: distances up to the diagonal
                if (pat == 2)
                    for (int c = 0; c < 3; ++c) {   // mostly empty columns
                        const int x = (int)(rng() % W);
                        for (int i = 0; i < 5; ++i) occ[(size_t)x * H + rng() % H] = 1;
                    }
                ++cases;
                fails += !check(occ, W, H, "large_side");
            }
    }
    printf("%d cases, %d mismatches\n", cases, fails);
    return fails != 0;
}
