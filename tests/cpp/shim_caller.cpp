// A C++ caller written against the reference's ranges:: API (RangeLib.h),
// built against include/RangeLib.h and librangelibc_gb300.so.
//
// usage: shim_caller <in.bin> <out.bin>
//   in.bin : int32 W, H; uint8 occ[W*H] (grid[x][y] at x*H+y); float world[6];
//            int32 n, na, K; float ins[n*3]; float angles[na]; float obs[na]; double table[K*K]
//   out.bin: float bl[n], rm[n], cddt[n], pcddt[n]; float ranges[n*na];
//            double eval[n], fused[n]; float dt[W*H]; float rmgpu_raw[n];
//            float glt[n]; uint16 lut[W*H*36]; float pair[n][2]; float radial[n*61];
//            float pcddt_from_json[n]
//   <out.bin>.json / <out.bin>.json7: the pruned table's serializeJson at 9 / 7 digits
#include "RangeLib.h"

#include <cstdio>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

using namespace ranges;

template <class T> static void rd(FILE* f, T* p, size_t n) {
    if (fread(p, sizeof(T), n, f) != n) throw std::runtime_error("short read");
}
template <class T> static void wr(FILE* f, const T* p, size_t n) { fwrite(p, sizeof(T), n, f); }

int main(int argc, char** argv) {
    if (argc != 3) return 2;
    FILE* f = fopen(argv[1], "rb");
    if (!f) return 2;
    int W, H, n, na, K;
    rd(f, &W, 1);
    rd(f, &H, 1);
    std::vector<uint8_t> occ((size_t)W * H);
    rd(f, occ.data(), occ.size());
    float world[6];
    rd(f, world, 6);
    rd(f, &n, 1);
    rd(f, &na, 1);
    rd(f, &K, 1);
    std::vector<float> ins((size_t)n * 3), angles(na), obs(na);
    std::vector<double> table((size_t)K * K);
    rd(f, ins.data(), ins.size());
    rd(f, angles.data(), na);
    rd(f, obs.data(), na);
    rd(f, table.data(), table.size());
    fclose(f);

    OMap map(W, H);
    for (int x = 0; x < W; ++x)
        for (int y = 0; y < H; ++y) map.grid[x][y] = occ[(size_t)x * H + y] != 0;
    map.world_scale = world[0];
    map.world_angle = world[1];
    map.world_origin_x = world[2];
    map.world_origin_y = world[3];
    map.world_sin_angle = world[4];
    map.world_cos_angle = world[5];

    std::vector<float> bl(n), rm(n), cd(n), pcd(n), ranges_((size_t)n * na), raw(n);
    std::vector<double> ev(n), fu(n);
    BresenhamsLine b(map, 150.0f);
    RayMarching r(map, 150.0f);
    CDDTCast c(map, 150.0f, 108);
    CDDTCast p(map, 150.0f, 108);
    p.prune(150.0f);
    RayMarchingGPU g(map, 150.0f);
    b.numpy_calc_range(ins.data(), bl.data(), n);
    r.numpy_calc_range(ins.data(), rm.data(), n);
    c.numpy_calc_range(ins.data(), cd.data(), n);
    p.numpy_calc_range(ins.data(), pcd.data(), n);
    r.numpy_calc_range_angles(ins.data(), angles.data(), ranges_.data(), n, na);
    r.set_sensor_model(table.data(), K);
    r.eval_sensor_model(obs.data(), ranges_.data(), ev.data(), na, n);
    r.calc_range_repeat_angles_eval_sensor_model(ins.data(), angles.data(), obs.data(), fu.data(), n, na);
    DistanceTransform dt(&map);
    g.calc_range_many(ins.data(), raw.data(), n);
    if (g.calc_range(1.0f, 1.0f, 0.0f) != -1.0f) return 3;
    if (c.compressed_lut().size() != 108) return 4;

    GiantLUTCast glt(map, 150.0f, 36);
    std::vector<float> gl(n), pr((size_t)n * 2), rad((size_t)n * 61, -7.0f);
    glt.numpy_calc_range(ins.data(), gl.data(), n);
    std::vector<uint16_t> lut = glt.lut();
    if (glt.lut_size() != (int)(lut.size() * sizeof(uint16_t))) return 6;
    for (int i = 0; i < n; ++i) {
        std::pair<float, float> q = c.calc_range_pair(ins[3 * i], ins[3 * i + 1], ins[3 * i + 2]);
        pr[2 * i] = q.first;
        pr[2 * i + 1] = q.second;
    }
    c.calc_range_many_radial_optimized(ins.data(), rad.data(), n, 61, -2.35619449f, 2.35619449f);

    // the pruned table through serializeJson / loadJson into an unpruned method
    std::stringstream js, js7;
    p.serializeJson(&js);
    p.serializeJson(&js7, 7);
    std::ofstream(std::string(argv[2]) + ".json") << js.str();
    std::ofstream(std::string(argv[2]) + ".json7") << js7.str();
    CDDTCast q(map, 150.0f, 108);
    q.loadJson(js.str());
    std::vector<float> qcd(n);
    q.numpy_calc_range(ins.data(), qcd.data(), n);

    FILE* o = fopen(argv[2], "wb");
    wr(o, bl.data(), n);
    wr(o, rm.data(), n);
    wr(o, cd.data(), n);
    wr(o, pcd.data(), n);
    wr(o, ranges_.data(), ranges_.size());
    wr(o, ev.data(), n);
    wr(o, fu.data(), n);
    for (int x = 0; x < W; ++x) wr(o, dt.grid[x].data(), H);
    wr(o, raw.data(), n);
    wr(o, gl.data(), n);
    wr(o, lut.data(), lut.size());
    wr(o, pr.data(), pr.size());
    wr(o, rad.data(), rad.size());
    wr(o, qcd.data(), n);
    fclose(o);
    // a bad call surfaces as an exception, not a crash
    try {
        r.eval_sensor_model(obs.data(), ranges_.data(), ev.data(), -1, n);
        return 5;
    } catch (const RangeLibError& e) {
    }
    // a table of another theta_discretization is refused
    try {
        CDDTCast other(map, 150.0f, 54);
        other.loadJson(js.str());
        return 7;
    } catch (const RangeLibError& e) {
    }
    return 0;
}
