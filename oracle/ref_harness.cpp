// Harness over the reference implementation -- TEST INFRASTRUCTURE.
//
// Compiled (oracle/Makefile, target `ref`) against the reference's own
// header-only sources where they are present, into oracle/_ref/.  It exposes
// the reference's classes through a C ABI so that the tests can (1) pin the
// C oracle against the reference and (2) generate the golden vectors under
// tests/golden/.  Nothing in the shipped library links it.
//
// Wrapped reference entry points (kctess5/range_libc, includes/RangeLib.h):
//   OMap(int, int) 143-156 + world fields 134-141, DistanceTransform 345-373,
//   BresenhamsLine 691-772, RayMarching 922-969, CDDTCast 971-1770 (+ prune),
//   RangeMethod::numpy_calc_range 439-480, numpy_calc_range_angles 482-520,
//   set_sensor_model 523-532, eval_sensor_model 533-555,
//   calc_range_repeat_angles_eval_sensor_model 558-612,
//   CDDTCast::calc_range_pair 1521-1615, calc_range_many_radial_optimized 616-676,
//   GiantLUTCast 1772-1904 (+ get_slice), CDDTCast::serializeJson 1690-1735.
#include "includes/RangeLib.h"

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <sstream>
#include <string>

using namespace ranges;

namespace {
struct RefMethod {
    int kind;  // 0 BL, 1 RM, 2 CDDT, 3 GLT
    RangeMethod* m;
    CDDTCast* cddt;
    GiantLUTCast* glt;
};
}  // namespace

extern "C" {

void* ref_map_create(const uint8_t* occ, int w, int h, float ws, float wa, float ox, float oy,
                     float wsin, float wcos) {
    OMap* map = new OMap(w, h);
    for (int x = 0; x < w; ++x)
        for (int y = 0; y < h; ++y) map->grid[x][y] = occ[(size_t)x * h + y] != 0;
    map->world_scale = ws;
    map->world_angle = wa;
    map->world_origin_x = ox;
    map->world_origin_y = oy;
    map->world_sin_angle = wsin;
    map->world_cos_angle = wcos;
    return map;
}

void ref_map_destroy(void* map) { delete static_cast<OMap*>(map); }

// Reference PNG loader (OMap(std::string, float), RangeLib.h:159-201).
// Returns a map handle or NULL; *w, *h receive the size.
void* ref_map_load_png(const char* path, float threshold, int* w, int* h) {
    OMap* map = new OMap(std::string(path), threshold);
    if (map->error()) { delete map; return nullptr; }
    *w = (int)map->width;
    *h = (int)map->height;
    map->world_scale = 1.0f; map->world_angle = 0.0f;
    map->world_origin_x = 0.0f; map->world_origin_y = 0.0f;
    map->world_sin_angle = 0.0f; map->world_cos_angle = 1.0f;
    return map;
}

void ref_map_grid(void* map, uint8_t* occ) {
    OMap* m = static_cast<OMap*>(map);
    for (unsigned x = 0; x < m->width; ++x)
        for (unsigned y = 0; y < m->height; ++y) occ[(size_t)x * m->height + y] = m->grid[x][y] ? 1 : 0;
}

void ref_dt(void* map, float* out) {
    OMap* m = static_cast<OMap*>(map);
    DistanceTransform dt(m);
    for (unsigned x = 0; x < dt.width; ++x)
        for (unsigned y = 0; y < dt.height; ++y) out[(size_t)x * dt.height + y] = dt.grid[x][y];
}

void ref_edge_map(void* map, uint8_t* out) {
    OMap* m = static_cast<OMap*>(map);
    OMap e = m->make_edge_map(true);
    for (unsigned x = 0; x < m->width; ++x)
        for (unsigned y = 0; y < m->height; ++y) out[(size_t)x * m->height + y] = e.grid[x][y] ? 1 : 0;
}

void* ref_method_create(void* map, int kind, float max_range, unsigned td) {
    OMap* m = static_cast<OMap*>(map);
    RefMethod* r = new RefMethod();
    r->kind = kind;
    r->cddt = nullptr;
    r->glt = nullptr;
    if (kind == 0) r->m = new BresenhamsLine(*m, max_range);
    else if (kind == 1) r->m = new RayMarching(*m, max_range);
    else if (kind == 3) { r->glt = new GiantLUTCast(*m, max_range, (int)td); r->m = r->glt; }
    else { r->cddt = new CDDTCast(*m, max_range, td); r->m = r->cddt; }
    return r;
}

void ref_method_destroy(void* h) {
    RefMethod* r = static_cast<RefMethod*>(h);
    delete r->m;
    delete r;
}

float ref_calc_range(void* h, float x, float y, float heading) {
    return static_cast<RefMethod*>(h)->m->calc_range(x, y, heading);
}

void ref_calc_range_many_raw(void* h, const float* ins, float* outs, int n) {
    RangeMethod* m = static_cast<RefMethod*>(h)->m;
    for (int i = 0; i < n; ++i) outs[i] = m->calc_range(ins[3 * i], ins[3 * i + 1], ins[3 * i + 2]);
}

void ref_numpy_calc_range(void* h, float* ins, float* outs, int n) {
    static_cast<RefMethod*>(h)->m->numpy_calc_range(ins, outs, n);
}

void ref_numpy_calc_range_angles(void* h, float* ins, float* angles, float* outs, int n, int na) {
    static_cast<RefMethod*>(h)->m->numpy_calc_range_angles(ins, angles, outs, n, na);
}

void ref_set_sensor_model(void* h, double* table, int k) {
    static_cast<RefMethod*>(h)->m->set_sensor_model(table, k);
}

void ref_eval_sensor_model(void* h, float* obs, float* ranges, double* outs, int rays, int particles) {
    static_cast<RefMethod*>(h)->m->eval_sensor_model(obs, ranges, outs, rays, particles);
}

void ref_fused(void* h, float* ins, float* angles, float* obs, double* weights, int n, int na) {
    static_cast<RefMethod*>(h)->m->calc_range_repeat_angles_eval_sensor_model(ins, angles, obs, weights, n, na);
}

void ref_cddt_prune(void* h, float max_range) {
    RefMethod* r = static_cast<RefMethod*>(h);
    if (r->cddt) r->cddt->prune(max_range);
}

// CDDT table shape: number of slices (td), bins per slice and total zeros.
long long ref_cddt_num_zeros(void* h) {
    CDDTCast* c = static_cast<RefMethod*>(h)->cddt;
    long long n = 0;
    for (auto& s : c->compressed_lut)
        for (auto& b : s) n += (long long)b.size();
    return n;
}

long long ref_cddt_num_bins(void* h) {
    CDDTCast* c = static_cast<RefMethod*>(h)->cddt;
    long long n = 0;
    for (auto& s : c->compressed_lut) n += (long long)s.size();
    return n;
}

// widths[td], trans[td], bin_len[num_bins], zeros[num_zeros]
void ref_cddt_export(void* h, int* widths, float* trans, long long* bin_len, float* zeros) {
    CDDTCast* c = static_cast<RefMethod*>(h)->cddt;
    long long b = 0, z = 0;
    for (size_t a = 0; a < c->compressed_lut.size(); ++a) {
        widths[a] = (int)c->compressed_lut[a].size();
        trans[a] = c->lut_translations[a];
        for (auto& bin : c->compressed_lut[a]) {
            bin_len[b++] = (long long)bin.size();
            for (float v : bin) zeros[z++] = v;
        }
    }
}

void ref_cddt_pair(void* h, float x, float y, float heading, float* r, float* r_inv) {
    std::pair<float, float> p = static_cast<RefMethod*>(h)->cddt->calc_range_pair(x, y, heading);
    *r = p.first;
    *r_inv = p.second;
}

void ref_cddt_radial(void* h, float* ins, float* outs, int n, int num_rays, float min_angle, float max_angle) {
    static_cast<RefMethod*>(h)->cddt->calc_range_many_radial_optimized(ins, outs, n, num_rays, min_angle, max_angle);
}

// the 16-bit LUT entries of angle bin `theta` as floats, out[x * height + y]
void ref_glt_slice(void* h, float theta, float* out) {
    DistanceTransform* d = static_cast<RefMethod*>(h)->glt->get_slice(theta);
    for (unsigned x = 0; x < d->width; ++x)
        for (unsigned y = 0; y < d->height; ++y) out[(size_t)x * d->height + y] = d->grid[x][y];
    delete d;
}

// CDDTCast::serializeJson: copies up to `cap` bytes of the document into buf and
// returns its full length (call with cap 0 to size the buffer)
long long ref_cddt_json(void* h, char* buf, long long cap) {
    std::stringstream ss;
    static_cast<RefMethod*>(h)->cddt->serializeJson(&ss);
    const std::string doc = ss.str();
    if (buf && cap > 0) std::memcpy(buf, doc.data(), std::min((size_t)cap, doc.size()));
    return (long long)doc.size();
}

}  // extern "C"
