// Host check of the correctly rounded sine/cosine of range_libc_gb300/csrc/rlc_trig.cuh.
//
//   trig_check scan LO HI STRIDE THREADS
//       every STRIDE-th float in [LO, HI): compares rlc_trig::sincos_cr with the float
//       rounding of the long double sinl/cosl (64 or 113 significand bits), and counts how
//       often the fast path defers to the double fallback and how often the host libm's
//       sinf/cosf differ from the correctly rounded values.
//   trig_check eval            reads float32 arguments on stdin, writes (sin, cos) pairs
//   trig_check diff N THREADS  N random (th, a) pairs per thread and family: sin and cos of
//       fl(th - a) through rlc_trig::sincos_diff (float pairs of th's and a's sin and cos, the
//       angle-difference formulas and a rounding check) against rlc_trig::sincos_cr, bit for bit
// Compile with -ffp-contract=off (no contraction: the device build uses -fmad=false).
#include "../../range_libc_gb300/csrc/rlc_trig.cuh"

#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <thread>
#include <vector>

static float nearest(long double v) { return (float)v; }

int main(int argc, char** argv) {
    if (argc >= 2 && !strcmp(argv[1], "eval")) {
        float x;
        while (fread(&x, 4, 1, stdin) == 1) {
            float sc[2];
            rlc_trig::sincos_cr(x, &sc[0], &sc[1]);
            fwrite(sc, 4, 2, stdout);
        }
        return 0;
    }
    if (argc >= 4 && !strcmp(argv[1], "diff")) {
        const long per = strtol(argv[2], nullptr, 10);
        const int nt = atoi(argv[3]) > 0 ? atoi(argv[3]) : 1;
        std::atomic<long> n{0}, bad{0}, fallback{0}, nopair{0};
        std::vector<std::thread> th;
        for (int t = 0; t < nt; ++t) {
            th.emplace_back([&, t]() {
                uint64_t st = 0x9E3779B97F4A7C15ull * (uint64_t)(t + 1);
                auto next = [&]() {
                    st ^= st << 13; st ^= st >> 7; st ^= st << 17;
                    return (double)(st >> 11) * 0x1p-53;
                };
                long ln = 0, lbad = 0, lfb = 0, lnp = 0;
                for (long i = 0; i < per; ++i) {
                    for (int fam = 0; fam < 4; ++fam) {
                        float hd, an;
                        if (fam == 0) {          // the workloads: grid headings, beams over 270 degrees
                            hd = (float)(-12.0 + 14.0 * next());
                            an = (float)(-2.4 + 4.8 * next());
                        } else if (fam == 1) {   // wide arguments
                            hd = (float)(-64.0 + 128.0 * next());
                            an = (float)(-64.0 + 128.0 * next());
                        } else if (fam == 2) {   // differences near multiples of pi / 2 (small sines or cosines)
                            an = (float)(-3.0 + 6.0 * next());
                            const int k = (int)(next() * 9.0) - 4;
                            hd = (float)((double)an + k * 1.5707963267948966 + (next() - 0.5) * 1e-3);
                        } else {                 // beams that nearly cancel the heading
                            an = (float)(-3.0 + 6.0 * next());
                            hd = an + (float)((next() - 0.5) * 0x1p-8);
                        }
                        rlc_trig::F2 ps, pc, bs, bc;
                        ++ln;
                        if (!rlc_trig::sincos_pairs(hd, &ps, &pc) || !rlc_trig::sincos_pairs(an, &bs, &bc)) {
                            ++lnp;
                            continue;
                        }
                        float s1, c1, s2, c2;
                        if (!rlc_trig::sincos_diff(hd, an, ps, pc, bs, bc, &s1, &c1)) {
                            ++lfb;
                            continue;
                        }
                        rlc_trig::sincos_cr(hd - an, &s2, &c2);
                        if (memcmp(&s1, &s2, 4) || memcmp(&c1, &c2, 4)) {
                            if (lbad < 5) fprintf(stderr, "mismatch th=%a a=%a: %a %a vs %a %a\n", hd, an, s1, c1, s2, c2);
                            ++lbad;
                        }
                    }
                }
                n += ln; bad += lbad; fallback += lfb; nopair += lnp;
            });
        }
        for (auto& x : th) x.join();
        printf("{\"n\": %ld, \"mismatch\": %ld, \"fallback\": %ld, \"no_pair\": %ld}\n", n.load(), bad.load(),
               fallback.load(), nopair.load());
        return bad.load() != 0;
    }
    if (argc < 6 || strcmp(argv[1], "scan")) {
        fprintf(stderr, "usage: trig_check scan LO HI STRIDE THREADS | trig_check eval | trig_check diff N THREADS\n");
        return 2;
    }
    const float lo = strtof(argv[2], nullptr), hi = strtof(argv[3], nullptr);
    const long stride = strtol(argv[4], nullptr, 10);
    const int nt = atoi(argv[5]);
    // walk the floats of [lo, hi) in bit order: negative ones by decreasing magnitude
    std::vector<uint32_t> segs;
    auto bits = [](float f) { uint32_t u; memcpy(&u, &f, 4); return u; };
    struct Seg { uint32_t a, b; };   // bit patterns [a, b) of one sign
    std::vector<Seg> s;
    if (lo < 0.0f) s.push_back({bits(hi < 0.0f ? -hi : 0.0f) | (hi < 0.0f ? 0u : 0x80000000u), bits(-lo) | 0x80000000u});
    if (hi > 0.0f) s.push_back({bits(lo > 0.0f ? lo : 0.0f), bits(hi)});
    if (lo < 0.0f && hi > 0.0f) s[0].a = 0x80000000u;
    std::atomic<long> n{0}, bad{0}, slow{0}, libm_s{0}, libm_c{0};
    std::vector<std::thread> th;
    for (int t = 0; t < nt; ++t) {
        th.emplace_back([&, t]() {
            long ln = 0, lbad = 0, lslow = 0, ls = 0, lc = 0;
            for (const Seg& g : s) {
                for (uint64_t u = (uint64_t)g.a + (uint64_t)t * stride; u < g.b; u += (uint64_t)nt * stride) {
                    float x;
                    const uint32_t v = (uint32_t)u;
                    memcpy(&x, &v, 4);
                    float sf, cf, s2, c2;
                    if (!rlc_trig::sincos_fast(x, &sf, &cf)) {
                        ++lslow;
                        rlc_trig::sincos_cr(x, &sf, &cf);
                    }
                    const float st = nearest(sinl((long double)x)), ct = nearest(cosl((long double)x));
                    ++ln;
                    if (memcmp(&sf, &st, 4) || memcmp(&cf, &ct, 4)) {
                        if (lbad < 5) fprintf(stderr, "mismatch x=%a: %a %a vs %a %a\n", x, sf, cf, st, ct);
                        ++lbad;
                    }
                    s2 = sinf(x);
                    c2 = cosf(x);
                    ls += memcmp(&s2, &st, 4) != 0;
                    lc += memcmp(&c2, &ct, 4) != 0;
                }
            }
            n += ln; bad += lbad; slow += lslow; libm_s += ls; libm_c += lc;
        });
    }
    for (auto& x : th) x.join();
    printf("{\"n\": %ld, \"mismatch\": %ld, \"fallback\": %ld, \"libm_sinf_not_nearest\": %ld, "
           "\"libm_cosf_not_nearest\": %ld}\n", n.load(), bad.load(), slow.load(), libm_s.load(), libm_c.load());
    return bad.load() != 0;
}
