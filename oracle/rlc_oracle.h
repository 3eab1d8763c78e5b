/*
 * CPU oracle for the range_libc ray-casting hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * algorithms (kctess5/range_libc, includes/RangeLib.h and the vendored
 * Felzenszwalb-Huttenlocher distance transform) that the test-suite, the
 * smoke check and the CPU-baseline leg of bench.py compare results with.
 * Nothing in the shipped library links or calls it.
 *
 * Parity is pinned two ways: against golden vectors produced by the
 * reference itself (tests/golden/) and, where the reference sources are
 * present, against the reference compiled from source (oracle/_ref).
 *
 * It must be compiled with strict IEEE float semantics: -O3
 * -ffp-contract=off, no -ffast-math, no -march=native.  Every float/double
 * mix below mirrors the reference expression it cites.
 *
 * Grid layout everywhere: occ[x * height + y] (the reference's grid[x][y],
 * x < width, y < height); the distance transform uses the same layout.
 */
#ifndef RLC_ORACLE_H
#define RLC_ORACLE_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_BL = 0, ORC_RM = 1, ORC_CDDT = 2, ORC_GLT = 3 };

/* World parameters of an OMap (RangeLib.h:134-141). */
typedef struct orc_world {
    float scale, angle, origin_x, origin_y, sin_angle, cos_angle;
} orc_world;

/* A CDDT table in CSR form: slice a has widths[a] bins; bin b of slice a
 * holds zeros[bin_start[slice_base[a] + b] .. bin_start[slice_base[a] + b + 1]). */
typedef struct orc_cddt {
    int width, height;
    const uint8_t* occ;      /* borrowed */
    float max_range;
    unsigned td;
    float td_div_2pi;        /* theta_discretization_div_M_2PI (float member) */
    float twopi_div_td;      /* M_2PI_div_theta_discretization (float member) */
    int* widths;             /* [td] */
    float* trans;            /* [td] */
    int64_t* slice_base;     /* [td + 1] first global bin of each slice */
    int64_t* bin_start;      /* [total_bins + 1] */
    float* zeros;            /* [bin_start[total_bins]] */
    int64_t total_bins;
} orc_cddt;

/* GiantLUTCast (RangeLib.h:1772-1904): lut[(x * height + y) * td + i], uint16. */
typedef struct orc_glt {
    int width, height;
    unsigned td;
    float max_range;
    float td_div_2pi;        /* theta_discretization_div_M_2PI (float member) */
    float twopi_div_td;      /* M_2PI_div_theta_discretization (float member) */
    float max_div_limits;    /* max_range / 65535 */
    float limits_div_max;    /* 65535 / max_range */
    uint16_t* lut;
} orc_glt;

/* A range method over one map. */
typedef struct orc_method {
    int kind;                /* ORC_BL, ORC_RM, ORC_CDDT */
    int width, height;
    const uint8_t* occ;      /* borrowed */
    const float* dt;         /* RM: borrowed distance transform */
    orc_cddt* cddt;          /* CDDT: borrowed table */
    float max_range;
    orc_world world;
    const double* table;     /* sensor model, K x K row-major (borrowed) */
    int K;
    orc_glt* glt;            /* GLT: borrowed table */
    const float* trig;       /* BL/RM: per-ray (cos, sin) used instead of the libm's by the batched
                                calls, ray-indexed like their outputs (NULL: cosf/sinf) */
} orc_method;

/* ---- map preprocessing ---- */
void orc_edt(const uint8_t* occ, int width, int height, float* dt_out);
void orc_edge_map(const uint8_t* occ, int width, int height, uint8_t* edge_out);

/* ---- single rays in the reference's calc_range(x, y, heading) space ---- */
float orc_rm_calc_range(const float* dt, int width, int height, float max_range,
                        float x, float y, float heading, int* steps);
float orc_rm_calc_range_trig(const float* dt, int width, int height, float max_range,
                             float x, float y, float c, float s, int* steps);
float orc_bl_calc_range(const uint8_t* occ, int width, int height, float max_range,
                        float x, float y, float heading, int* steps);
float orc_bl_calc_range_trig(const uint8_t* occ, int width, int height, float max_range,
                             float x, float y, float c, float s, int* steps);

/* ---- CDDT ---- */
orc_cddt* orc_cddt_build(const uint8_t* occ, int width, int height, float max_range, unsigned td);
void orc_cddt_prune(orc_cddt* c, float max_range);
void orc_cddt_free(orc_cddt* c);
void orc_cddt_discretize(const orc_cddt* c, float theta, int* binned, float* discrete, int* flipped);
float orc_cddt_calc_range(const orc_cddt* c, float x, float y, float heading, int* probes);
int64_t orc_cddt_num_zeros(const orc_cddt* c);
/* Replace the table of c by a caller-provided CSR table (same td/widths). */
int orc_cddt_load(orc_cddt* c, const int* widths, const float* trans,
                  const int64_t* bin_len, const float* zeros, int64_t nzeros);

/* calc_range_pair (RangeLib.h:1521-1615): ranges at heading and heading + pi from one bin search. */
void orc_cddt_calc_range_pair(const orc_cddt* c, float x, float y, float heading, float* r, float* r_inv);
/* calc_range_many_radial_optimized (RangeLib.h:616-676), world frame, m->kind == ORC_CDDT.
 * Positions of a particle's row that the reference does not write are left as they are;
 * writes that the reference sends past the row (into the next particle's row, which that
 * particle then overwrites, or past the array) are dropped. */
void orc_cddt_radial(const orc_method* m, const float* ins, float* outs, int n, int num_rays,
                     float min_angle, float max_angle);

/* ---- GiantLUTCast ---- */
/* Build from the distance transform: one RayMarching cast from each cell corner (x, y) at each
 * of the td angles, clamped to max_range and stored as uint16 (RangeLib.h:1782-1818). */
orc_glt* orc_glt_build(const float* dt, int width, int height, float max_range, unsigned td, int nthreads);
void orc_glt_free(orc_glt* g);
int orc_glt_discretize(const orc_glt* g, float theta);
float orc_glt_calc_range(const orc_glt* g, float x, float y, float heading);

/* ---- batched RangeMethod API (RangeLib.h:439-612) ---- */
float orc_method_calc_range(const orc_method* m, float x, float y, float heading, int* steps);
void orc_numpy_calc_range(const orc_method* m, const float* ins, float* outs, int n, int nthreads);
void orc_calc_range_many_raw(const orc_method* m, const float* ins, float* outs, int n, int nthreads);
void orc_numpy_calc_range_angles(const orc_method* m, const float* ins, const float* angles,
                                 float* outs, int n, int na, int nthreads);
void orc_eval_sensor_model(const orc_method* m, const float* obs, const float* ranges,
                           double* outs, int rays_per_particle, int particles, int nthreads);
void orc_calc_range_repeat_angles_eval_sensor_model(const orc_method* m, const float* ins,
                                                    const float* angles, const float* obs,
                                                    double* weights, int n, int na, int nthreads);

/* Parity helpers: the calc_range-space pose and heading of each ray of the
 * world-frame APIs, exactly as the reference computes them.  xyh gets
 * (x, y, heading) per ray; trig gets (cosf(heading), sinf(heading)). */
void orc_world_rays(const orc_world* w, const float* ins, const float* angles, int n, int na,
                    float* xyh, float* trig);
/* Mean march steps per ray over the world-frame rays (for algorithmic bytes). */
double orc_mean_steps(const orc_method* m, const float* ins, const float* angles, int n, int na);

#ifdef __cplusplus
}
#endif
#endif
