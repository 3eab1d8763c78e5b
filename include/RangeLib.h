// RangeLib.h -- C++ API of the GB300 ray-casting library.
//
// Mirrors the reference's header-only `namespace ranges` (kctess5/range_libc,
// includes/RangeLib.h:120-1905) for the batched hot path: the same class
// names, constructors and methods, the same argument meaning.  Every method
// runs on the GPU through the C ABI (rangelibc.h); link with
// -lrangelibc_gb300.  There is no CPU path.
//
// Differences a caller may notice:
//  * errors throw ranges::RangeLibError (std::runtime_error) instead of
//    printing (the reference prints, throws std::string or invokes UB);
//  * CDDTCast::serializeJson prints 9 significant digits by default (the
//    reference prints 7, which does not restore every float) and loadJson
//    reads the document back; serializeYaml and saveTrace are not provided.
#ifndef RANGELIB_GB300_H
#define RANGELIB_GB300_H

#include "rangelibc.h"

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace ranges {

struct RangeLibError : std::runtime_error {
    int code;
    RangeLibError(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

inline void check(int rc) {
    if (rc != RLC_OK) throw RangeLibError(rc, rlc_last_error());
}

// OMap (RangeLib.h:121-322): grid[x][y], x < width, y < height, plus the ROS world parameters.
struct OMap {
    bool has_error;
    unsigned width;
    unsigned height;
    std::vector<std::vector<bool> > grid;
    std::string fn;
    float world_scale = 1.0f;
    float world_angle = 0.0f;
    float world_origin_x = 0.0f;
    float world_origin_y = 0.0f;
    float world_sin_angle = 0.0f;
    float world_cos_angle = 1.0f;

    OMap(int w, int h)
        : has_error(false), width((unsigned)w), height((unsigned)h),
          grid((size_t)w, std::vector<bool>((size_t)h, false)) {}

    // OMap(std::string[, float]) (RangeLib.h:158-201): a PNG map; pixel (x, y) is occupied when
    // (int)rgb2gray(r, g, b) < threshold.  A file that cannot be read prints the error and sets
    // has_error, as in the reference.
    explicit OMap(const std::string& filename, float threshold = 128.0f)
        : has_error(false), width(0), height(0), fn(filename) {
        int w = 0, h = 0;
        int rc = rlc_png_occupancy(filename.c_str(), threshold, nullptr, &w, &h);
        std::vector<uint8_t> occ;
        if (rc == RLC_OK) {
            occ.resize((size_t)w * h);
            rc = rlc_png_occupancy(filename.c_str(), threshold, occ.data(), &w, &h);
        }
        if (rc != RLC_OK) {
            std::printf("ERROR %d: %s\n", rc, rlc_last_error());
            has_error = true;
            return;
        }
        width = (unsigned)w;
        height = (unsigned)h;
        grid.assign(width, std::vector<bool>(height, false));
        for (unsigned x = 0; x < width; ++x)
            for (unsigned y = 0; y < height; ++y) grid[x][y] = occ[(size_t)x * height + y] != 0;
    }

    // save (RangeLib.h:263-291): occupied black, free white; true when the file could not be written
    bool save(const std::string& filename) {
        const std::vector<uint8_t> occ = occupancy();
        const int rc = rlc_png_save_occupancy(filename.c_str(), occ.data(), (int)width, (int)height);
        if (rc != RLC_OK) std::cout << "encoder error " << rc << ": " << rlc_last_error() << std::endl;
        return rc != RLC_OK;
    }

    bool get(int x, int y) { return grid[x][y]; }
    bool isOccupied(int x, int y) {
        if (x < 0 || x >= (int)width || y < 0 || y >= (int)height) return false;
        return grid[x][y];
    }
    bool isOccupiedNT(int x, int y) { return grid[x][y]; }
    bool error() { return has_error; }
    int memory() { return (int)(sizeof(bool) * width * height); }

    // occ[x * height + y], the C ABI's layout
    std::vector<uint8_t> occupancy() const {
        std::vector<uint8_t> o((size_t)width * height);
        for (unsigned x = 0; x < width; ++x)
            for (unsigned y = 0; y < height; ++y) o[(size_t)x * height + y] = grid[x][y] ? 1 : 0;
        return o;
    }

    // make_edge_map(true) (RangeLib.h:293-312), computed on the GPU
    OMap make_edge_map(bool count_corners) {
        if (!count_corners) throw RangeLibError(RLC_ERR_ARG, "make_edge_map: only the 8-neighbour outline is provided");
        std::vector<uint8_t> occ = occupancy(), edge(occ.size());
        rlc_map* h = nullptr;
        check(rlc_map_create(occ.data(), (int)width, (int)height, &h));
        int rc = rlc_map_edge_map(h, edge.data());
        rlc_map_destroy(h);
        check(rc);
        OMap e((int)width, (int)height);
        for (unsigned x = 0; x < width; ++x)
            for (unsigned y = 0; y < height; ++y) e.grid[x][y] = edge[(size_t)x * height + y] != 0;
        return e;
    }
};

// DistanceTransform(OMap*) (RangeLib.h:324-410), computed on the GPU.
struct DistanceTransform {
    unsigned width = 0;
    unsigned height = 0;
    std::vector<std::vector<float> > grid;

    DistanceTransform() {}
    explicit DistanceTransform(OMap* map) : width(map->width), height(map->height) {
        std::vector<uint8_t> occ = map->occupancy();
        std::vector<float> dt(occ.size());
        rlc_map* h = nullptr;
        check(rlc_map_create(occ.data(), (int)width, (int)height, &h));
        int rc = rlc_map_distance_transform(h, dt.data());
        rlc_map_destroy(h);
        check(rc);
        grid.assign(width, std::vector<float>(height));
        for (unsigned x = 0; x < width; ++x)
            for (unsigned y = 0; y < height; ++y) grid[x][y] = dt[(size_t)x * height + y];
    }
    float get(int x, int y) { return grid[x][y]; }
    int memory() { return (int)(width * height * sizeof(float)); }
};

// RangeMethod (RangeLib.h:412-689).  Methods take the map by value, as in
// the reference: later changes to the caller's OMap are not seen.
class RangeMethod {
public:
    RangeMethod(OMap m, float mr, int kind, unsigned td = 0) : map(std::move(m)), max_range(mr) {
        std::vector<uint8_t> occ = map.occupancy();
        check(rlc_map_create(occ.data(), (int)map.width, (int)map.height, &hmap));
        check(rlc_map_set_world(hmap, map.world_scale, map.world_angle, map.world_origin_x, map.world_origin_y,
                                map.world_sin_angle, map.world_cos_angle));
        check(rlc_method_create(hmap, kind, mr, td, &h));
    }
    virtual ~RangeMethod() {
        if (h) rlc_method_destroy(h);
        if (hmap) rlc_map_destroy(hmap);
    }
    RangeMethod(const RangeMethod&) = delete;
    RangeMethod& operator=(const RangeMethod&) = delete;

    virtual float calc_range(float x, float y, float heading) {
        float out = 0.0f;
        check(rlc_calc_range(h, x, y, heading, &out));
        return out;
    }
    virtual OMap* getMap() { return &map; }
    float maxRange() { return max_range; }

    void numpy_calc_range(float* ins, float* outs, int num_casts) {
        check(rlc_calc_range_many(h, ins, outs, num_casts, 0, nullptr));
    }
    void numpy_calc_range_angles(float* ins, float* angles, float* outs, int num_particles, int num_angles) {
        check(rlc_calc_range_repeat_angles(h, ins, angles, outs, num_particles, num_angles, 0, nullptr));
    }
    void set_sensor_model(double* table, int table_width) { check(rlc_set_sensor_model(h, table, table_width)); }
    void eval_sensor_model(float* obs, float* ranges, double* outs, int rays_per_particle, int particles) {
        check(rlc_eval_sensor_model(h, obs, ranges, outs, rays_per_particle, particles, 0, nullptr));
    }
    void calc_range_repeat_angles_eval_sensor_model(float* ins, float* angles, float* obs, double* weights,
                                                    int num_particles, int num_angles) {
        check(rlc_calc_range_repeat_angles_eval_sensor_model(h, ins, angles, obs, weights, num_particles, num_angles,
                                                             0, nullptr));
    }
    void saveTrace(std::string) {
        std::cout << "WARNING: trace map not generated, must compile with trace support enabled." << std::endl;
    }

    rlc_method* handle() { return h; }

protected:
    OMap map;
    float max_range;
    rlc_map* hmap = nullptr;
    rlc_method* h = nullptr;
};

class BresenhamsLine : public RangeMethod {
public:
    BresenhamsLine(OMap m, float mr) : RangeMethod(std::move(m), mr, RLC_BL) {}
    int memory() { return map.memory(); }
};

class RayMarching : public RangeMethod {
public:
    RayMarching(OMap m, float mr) : RangeMethod(std::move(m), mr, RLC_RM) {}
};

class CDDTCast : public RangeMethod {
public:
    CDDTCast(OMap m, float mr, unsigned int td) : RangeMethod(std::move(m), mr, RLC_CDDT, td), theta_discretization(td) {}
    void prune(float max_range_) { check(rlc_cddt_prune(h, max_range_)); }
    // compressed_lut[theta][bin] -> zero points, and lut_translations (RangeLib.h:1742-1748)
    std::vector<std::vector<std::vector<float> > > compressed_lut() {
        int64_t nb = 0, nz = 0;
        check(rlc_cddt_table_size(h, &nb, &nz));
        std::vector<int> widths(theta_discretization);
        std::vector<float> trans(theta_discretization), zeros((size_t)nz);
        std::vector<int64_t> len((size_t)nb);
        check(rlc_cddt_table_export(h, widths.data(), trans.data(), len.data(), zeros.data()));
        std::vector<std::vector<std::vector<float> > > lut(theta_discretization);
        size_t b = 0, z = 0;
        for (unsigned a = 0; a < theta_discretization; ++a) {
            lut[a].resize((size_t)widths[a]);
            for (int i = 0; i < widths[a]; ++i, ++b) {
                lut[a][i].assign(zeros.begin() + z, zeros.begin() + z + len[b]);
                z += (size_t)len[b];
            }
        }
        return lut;
    }
    // calc_range_pair (RangeLib.h:1521-1615): ranges at heading and heading + pi
    std::pair<float, float> calc_range_pair(float x, float y, float heading) {
        float r = 0.0f, ri = 0.0f;
        check(rlc_cddt_calc_range_pair(h, x, y, heading, &r, &ri));
        return std::make_pair(r, ri);
    }
    // calc_range_many_radial_optimized (RangeLib.h:616-676)
    void calc_range_many_radial_optimized(float* ins, float* outs, int num_particles, int num_rays, float min_angle,
                                          float max_angle) {
        check(rlc_cddt_calc_range_many_radial(h, ins, outs, num_particles, num_rays, min_angle, max_angle, 0,
                                              nullptr));
    }
    std::vector<float> lut_translations() {
        std::vector<int> widths(theta_discretization);
        std::vector<float> trans(theta_discretization);
        check(rlc_cddt_table_export(h, widths.data(), trans.data(), nullptr, nullptr));
        return trans;
    }

    // serializeJson (RangeLib.h:1690-1735): the reference's document -- keys, nesting, line
    // breaks, the comma after the map's data array -- with `precision` significant digits.  The
    // reference prints 7, which does not restore every float; 9 (the default) does, so loadJson
    // gives the table back bit for bit.  precision 7 reproduces the reference's text exactly.
    void serializeJson(std::stringstream* ss, int precision = 9) {
        const std::vector<std::vector<std::vector<float> > > lut = compressed_lut();
        const std::vector<float> trans = lut_translations();
        const std::streamsize old = ss->precision(precision);
        auto floats = [ss](const std::vector<float>& v) {
            (*ss) << "[";
            for (size_t i = 0; i < v.size(); ++i) (*ss) << (i ? "," : "") << v[i];
            (*ss) << "]";
        };
        (*ss) << "{\"cddt\": {\n  \"theta_discretization\": " << theta_discretization << ",\n";
        (*ss) << "  \"lut_translations\": ";
        floats(trans);
        (*ss) << ",\n  \"max_range\":" << max_range << ",\n  \"map\": {\n";
        (*ss) << "    \"path\": \"" << map.fn << "\",\n    \"width\": " << map.width << ",\n    \"height\": "
              << map.height << ",\n    \"data\": [";
        for (unsigned x = 0; x < map.width; ++x) {
            (*ss) << (x ? ",[" : "[");
            for (unsigned y = 0; y < map.height; ++y) (*ss) << (y ? "," : "") << (map.grid[x][y] ? '1' : '0');
            (*ss) << "]";
        }
        (*ss) << "],\n  },\n  \"compressed_lut\": [\n";
        const float step = (float)(6.28318530718 / (double)(float)theta_discretization);
        for (unsigned a = 0; a < theta_discretization; ++a) {
            const float theta = (float)a * step;
            (*ss) << "    {\n      \"theta\": " << theta << ",\n      \"zeros\": [";
            for (size_t i = 0; i < lut[a].size(); ++i) {
                if (i) (*ss) << ",";
                floats(lut[a][i]);
            }
            (*ss) << "]\n    }" << (a + 1 == theta_discretization ? "\n" : ",\n");
        }
        (*ss) << "  ]\n}}\n";
        ss->precision(old);
    }

    // loadJson: replace the table by the one in a serializeJson document (this library's or the
    // reference's) written for a map of the same size and the same theta_discretization
    void loadJson(const std::string& doc) {
        const char* s = doc.c_str();
        auto after = [&](const char* from, const char* key) {
            const char* p = std::strstr(from, key);
            if (!p) throw RangeLibError(RLC_ERR_ARG, std::string("loadJson: missing ") + key);
            return p + std::strlen(key);
        };
        auto skip = [](const char* p) {
            while (*p == ' ' || *p == '\n' || *p == '\r' || *p == '\t' || *p == ':' || *p == ',') ++p;
            return p;
        };
        auto floats = [&](const char*& p, std::vector<float>& out) {   // "[v, ...]"
            p = skip(p);
            if (*p != '[') throw RangeLibError(RLC_ERR_ARG, "loadJson: expected '['");
            p = skip(p + 1);
            while (*p != ']') {
                char* end = nullptr;
                out.push_back(std::strtof(p, &end));
                if (end == p) throw RangeLibError(RLC_ERR_ARG, "loadJson: bad number");
                p = skip(end);
            }
            ++p;
        };
        const char* p = after(s, "\"theta_discretization\"");
        if (std::strtoul(skip(p), nullptr, 10) != theta_discretization)
            throw RangeLibError(RLC_ERR_ARG, "loadJson: another theta_discretization");
        p = after(s, "\"width\"");
        const unsigned long w = std::strtoul(skip(p), nullptr, 10);
        p = after(s, "\"height\"");
        if (w != map.width || std::strtoul(skip(p), nullptr, 10) != map.height)
            throw RangeLibError(RLC_ERR_ARG, "loadJson: table of a map of another size");
        std::vector<float> trans, zeros;
        p = after(s, "\"lut_translations\"");
        floats(p, trans);
        if (trans.size() != theta_discretization) throw RangeLibError(RLC_ERR_ARG, "loadJson: lut_translations");
        int64_t nb = 0, nz = 0;
        check(rlc_cddt_table_size(h, &nb, &nz));
        std::vector<int> widths(theta_discretization);
        std::vector<float> cur(theta_discretization);
        check(rlc_cddt_table_export(h, widths.data(), cur.data(), nullptr, nullptr));
        std::vector<int64_t> len;
        p = after(s, "\"compressed_lut\"");
        for (unsigned a = 0; a < theta_discretization; ++a) {
            p = skip(after(p, "\"zeros\""));
            if (*p != '[') throw RangeLibError(RLC_ERR_ARG, "loadJson: expected '['");
            p = skip(p + 1);
            int bins = 0;
            while (*p != ']') {
                const size_t before = zeros.size();
                floats(p, zeros);
                len.push_back((int64_t)(zeros.size() - before));
                ++bins;
                p = skip(p);
            }
            ++p;
            if (bins != widths[a]) throw RangeLibError(RLC_ERR_ARG, "loadJson: slice widths differ from this map's");
        }
        check(rlc_cddt_table_load(h, trans.data(), len.data(), zeros.data(), (int64_t)zeros.size()));
    }
    unsigned int theta_discretization;
};

// GiantLUTCast (RangeLib.h:1772-1904): the 16-bit table is built on the GPU
class GiantLUTCast : public RangeMethod {
public:
    GiantLUTCast(OMap m, float mr, int td) : RangeMethod(std::move(m), mr, RLC_GLT, (unsigned)td), theta_discretization(td) {}
    int lut_size() { return (int)(map.width * map.height * (unsigned)theta_discretization * sizeof(uint16_t)); }
    int memory() { return lut_size(); }
    // the table, giant_lut[x][y][i] at [(x * height + y) * td + i]
    std::vector<uint16_t> lut() {
        std::vector<uint16_t> t((size_t)map.width * map.height * theta_discretization);
        check(rlc_glt_table(h, t.data()));
        return t;
    }
    int theta_discretization;
};

class RayMarchingGPU : public RangeMethod {
public:
    RayMarchingGPU(OMap m, float mr) : RangeMethod(std::move(m), mr, RLC_RMGPU) {}
    // RangeLib.h:800-807: single queries are not served by the GPU class
    float calc_range(float, float, float) override {
        std::cout << "Do not call calc_range on RayMarchingGPU, requires batched queries" << std::endl;
        return -1.0f;
    }
    // RangeLib.h:835-846: no world transform
    void calc_range_many(float* ins, float* outs, int num_casts) {
        check(rlc_calc_range_many(h, ins, outs, num_casts, RLC_NO_WORLD, nullptr));
    }
};

}  // namespace ranges

#endif  // RANGELIB_GB300_H
