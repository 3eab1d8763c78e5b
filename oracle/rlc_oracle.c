/*
 * CPU oracle for the range_libc ray-casting hot path -- TEST INFRASTRUCTURE.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use
 * this file, always as the oracle that results are compared with or as the
 * timed CPU baseline.  It is a
 * restatement in plain C of kctess5/range_libc (cited as RangeLib.h:<line>,
 * distance_transform.h:<line>, RangeUtils.h:<line>).  Build flags must keep
 * strict IEEE semantics: -O3 -ffp-contract=off (see oracle/Makefile).
 *
 * Conventions where the reference is undefined (documented, shared with the
 * CUDA library so both stay comparable):
 *  - float->int conversions saturate and map NaN to 0 (what cvt.rzi does);
 *    poses or headings that are NaN return max_range.
 *  - CDDT: a query cell outside the grid counts as free; the forward
 *    binary-search read one past the end of a bin (RangeLib.h:1480-1481 when
 *    x equals the last zero point) returns 0; prune's linear search that
 *    finds nothing (RangeLib.h:1242-1247, uninitialised index) reuses the
 *    index last assigned in the slice (see orc_cddt_prune).
 *  - sensor model: a NaN observation or range indexes bin 0.
 */
#include "rlc_oracle.h"

#include <float.h>
#include <limits.h>
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#define ORC_EPSILON 0.00001          /* RangeLib.h:60 _EPSILON (double) */
#define ORC_M_2PI 6.28318530718      /* RangeLib.h:61 M_2PI (double) */
#define ORC_M_PI 3.14159265358979323846
#define ORC_BSEARCH_THRESHOLD 64     /* RangeLib.h:62 */
#define ORC_STEP_COEFF 0.999f        /* RangeLib.h:968 step_coeff (float member) */
#define ORC_MAX_WRAP 100000          /* bound on discretize_theta's wrap loops */

/* float -> int with C truncation; saturating, NaN -> 0 (cvt.rzi.s32.f32). */
static inline int f2i(float v) {
    if (v != v) return 0;
    if (v >= 2147483648.0f) return INT_MAX;
    if (v <= -2147483904.0f) return INT_MIN;
    return (int)v;
}

/* std::max / std::min as the reference instantiates them. */
static inline float ref_maxf(float a, float b) { return (a < b) ? b : a; }
static inline float ref_minf(float a, float b) { return (b < a) ? b : a; }

/* ------------------------------------------------------------------ */
/* parallel-for over [0, n) in contiguous slices                        */
/* ------------------------------------------------------------------ */
typedef void (*orc_range_fn)(void* ctx, int lo, int hi);
typedef struct { orc_range_fn fn; void* ctx; int lo, hi; } orc_task;
static void* orc_task_main(void* p) { orc_task* t = (orc_task*)p; t->fn(t->ctx, t->lo, t->hi); return NULL; }

static void orc_parallel(orc_range_fn fn, void* ctx, int n, int nthreads) {
    if (nthreads <= 1 || n < 2 * nthreads) { fn(ctx, 0, n); return; }
    if (nthreads > 256) nthreads = 256;
    pthread_t th[256];
    orc_task tasks[256];
    int started[256];
    for (int t = 0; t < nthreads; ++t) {
        tasks[t].fn = fn; tasks[t].ctx = ctx;
        tasks[t].lo = (int)((int64_t)n * t / nthreads);
        tasks[t].hi = (int)((int64_t)n * (t + 1) / nthreads);
        started[t] = (t > 0) && pthread_create(&th[t], NULL, orc_task_main, &tasks[t]) == 0;
    }
    fn(ctx, tasks[0].lo, tasks[0].hi);
    for (int t = 1; t < nthreads; ++t) {
        if (started[t]) pthread_join(th[t], NULL);
        else fn(ctx, tasks[t].lo, tasks[t].hi);
    }
}

/* ------------------------------------------------------------------ */
/* Distance transform: Felzenszwalb & Huttenlocher lower envelope        */
/* (distance_transform.h:984-1030), per axis, then sqrt (1102-1125).     */
/* ------------------------------------------------------------------ */
static void fh_line(const float* f, ptrdiff_t fs, float* D, ptrdiff_t ds, size_t n,
                    size_t* v, double* z) {
    if (n == 0) return;
    if (n == 1) { D[0] = f[0]; return; }
    size_t k = 0;
    v[0] = 0;
    z[0] = -DBL_MAX;
    z[1] = DBL_MAX;
    for (size_t q = 1; q < n; ++q) {
        double s;
        ++k;
        do {
            --k;
            /* (f[q] + q*q) is a float sum; the right operand is cast to double */
            float fq = f[q * fs] + (float)(q * q);
            float fv = f[v[k] * fs] + (float)(v[k] * v[k]);
            s = ((double)fq - (double)fv) / ((double)(2 * q) - (double)(2 * v[k]));
        } while (s <= z[k]);
        ++k;
        v[k] = q;
        z[k] = s;
        z[k + 1] = DBL_MAX;
    }
    k = 0;
    for (size_t q = 0; q < n; ++q) {
        while (z[k + 1] < (double)q) ++k;
        float dq = (float)q - (float)v[k];
        D[q * ds] = f[v[k] * fs] + dq * dq;
    }
}

/* RangeLib.h:345-373: f = 0 on occupied cells, FLT_MAX elsewhere; slice 0
 * fixes x (lines along y), slice 1 fixes y (lines along x). */
void orc_edt(const uint8_t* occ, int width, int height, float* dt_out) {
    size_t W = (size_t)width, H = (size_t)height, N = W * H;
    if (N == 0) return;
    float* f = (float*)malloc(N * sizeof(float));
    float* g = (float*)malloc(N * sizeof(float));
    size_t nmax = W > H ? W : H;
    size_t* v = (size_t*)malloc(nmax * sizeof(size_t));
    double* z = (double*)malloc((nmax + 1) * sizeof(double));
    for (size_t i = 0; i < N; ++i) f[i] = occ[i] ? 0.0f : FLT_MAX;
    for (size_t x = 0; x < W; ++x) fh_line(f + x * H, 1, g + x * H, 1, H, v, z);
    for (size_t y = 0; y < H; ++y) fh_line(g + y, (ptrdiff_t)H, f + y, (ptrdiff_t)H, W, v, z);
    for (size_t i = 0; i < N; ++i) dt_out[i] = sqrtf(f[i]);
    free(f); free(g); free(v); free(z);
}

/* RangeLib.h:293-312 with utils::outline(x, y, true), RangeUtils.h:36-52. */
void orc_edge_map(const uint8_t* occ, int width, int height, uint8_t* edge_out) {
    static const int nb[8][2] = {{1, 0}, {-1, 0}, {0, 1}, {0, -1}, {1, 1}, {-1, 1}, {1, -1}, {-1, -1}};
    for (int x = 0; x < width; ++x)
        for (int y = 0; y < height; ++y) {
            size_t i = (size_t)x * height + y;
            edge_out[i] = 0;
            if (!occ[i]) continue;
            for (int k = 0; k < 8; ++k) {
                int cx = x + nb[k][0], cy = y + nb[k][1];
                if (0 <= cx && 0 <= cy && cx < width && cy < height &&
                    !occ[(size_t)cx * height + cy]) { edge_out[i] = 1; break; }
            }
        }
}

/* ------------------------------------------------------------------ */
/* Ray marching, RangeLib.h:927-962                                      */
/* ------------------------------------------------------------------ */
float orc_rm_calc_range_trig(const float* dt, int width, int height, float max_range,
                             float x, float y, float c, float s, int* steps) {
    float x0 = x, y0 = y;
    int n = 0;
    float t = 0.0f;
    float out = max_range;
    if (x0 != x0 || y0 != y0 || c != c || s != s) goto done;
    while (t < max_range) {
        int px = f2i(x0 + c * t);
        int py = f2i(y0 + s * t);
        if (px >= width || px < 0 || py < 0 || py >= height) { out = max_range; goto done; }
        float d = dt[(size_t)px * height + py];
        ++n;
        if (d <= 0.0f) {
            float xd = (float)px - x0;
            float yd = (float)py - y0;
            out = sqrtf(xd * xd + yd * yd);
            goto done;
        }
        t += ref_maxf(d * ORC_STEP_COEFF, 1.0f);
    }
done:
    if (steps) *steps = n;
    return out;
}

float orc_rm_calc_range(const float* dt, int width, int height, float max_range,
                        float x, float y, float heading, int* steps) {
    return orc_rm_calc_range_trig(dt, width, height, max_range, x, y, cosf(heading), sinf(heading), steps);
}

/* ------------------------------------------------------------------ */
/* Bresenham's line, RangeLib.h:696-769                                  */
/* ------------------------------------------------------------------ */
static inline int occ_at(const uint8_t* occ, int width, int height, int x, int y) {
    if (x < 0 || x >= width || y < 0 || y >= height) return 0;   /* isOccupied, RangeLib.h:203-210 */
    return occ[(size_t)x * height + y] != 0;
}

float orc_bl_calc_range_trig(const uint8_t* occ, int width, int height, float max_range,
                             float x, float y, float c, float s, int* steps) {
    int n = 0;
    float out = max_range;
    if (x != x || y != y) goto done;
    if (occ_at(occ, width, height, f2i(x), f2i(y))) { out = 0.0f; goto done; }
    if (c != c || s != s) goto done;   /* the reference loops forever on a NaN heading */
    {
        float x0 = y, y0 = x;
        float x1 = y + max_range * s;
        float y1 = x + max_range * c;
        int steep = fabsf(y1 - y0) > fabsf(x1 - x0);
        if (steep) {
            float tmp = x0; x0 = y0; y0 = tmp;
            tmp = x1; x1 = y1; y1 = tmp;
        }
        float deltax = fabsf(x1 - x0);
        float deltay = fabsf(y1 - y0);
        float error = 0.0f;
        float deltaerr = deltay;
        float _x = x0, _y = y0;
        int xstep = (x0 < x1) ? 1 : -1;
        int ystep = (y0 < y1) ? 1 : -1;
        float fw = (float)width, fh = (float)height;
        /* the reference loop ends after |x1-x0|+2 steps unless (int)_x never
         * equals the end: above 2^24 float +-1 no longer moves _x, and a start
         * whose fraction is 1 - ulp rounds up across a power of two and skips
         * that integer (999.99994 + 24 -> 1025.0); the reference then never
         * terminates, the bound returns max_range */
        long bound = (long)(deltax < 1e9f ? deltax : 1e9f) + 4;
        while (f2i(_x) != f2i(x1 + (float)xstep)) {
            if (n > bound) { out = max_range; goto done; }
            _x += (float)xstep;
            error += deltaerr;
            ++n;
            if ((double)error * 2.00 >= (double)deltax) {
                _y += (float)ystep;
                error -= deltax;
            }
            if (!steep) {
                if (0 <= _y && _y < fw && 0 <= _x && _x < fh && occ_at(occ, width, height, f2i(_y), f2i(_x))) {
                    float xd = _x - x0, yd = _y - y0;
                    out = sqrtf(xd * xd + yd * yd);
                    goto done;
                }
            } else {
                if (0 <= _x && _x < fw && 0 <= _y && _y < fh && occ_at(occ, width, height, f2i(_x), f2i(_y))) {
                    float xd = _x - x0, yd = _y - y0;
                    out = sqrtf(xd * xd + yd * yd);
                    goto done;
                }
            }
        }
    }
done:
    if (steps) *steps = n;
    return out;
}

float orc_bl_calc_range(const uint8_t* occ, int width, int height, float max_range,
                        float x, float y, float heading, int* steps) {
    return orc_bl_calc_range_trig(occ, width, height, max_range, x, y, cosf(heading), sinf(heading), steps);
}

/* ------------------------------------------------------------------ */
/* CDDT, RangeLib.h:974-1516                                             */
/* ------------------------------------------------------------------ */
static int cmp_float(const void* a, const void* b) {
    float fa = *(const float*)a, fb = *(const float*)b;
    return (fa < fb) ? -1 : (fb < fa) ? 1 : 0;
}

static void cddt_alloc_slices(orc_cddt* c) {
    c->slice_base = (int64_t*)malloc((c->td + 1) * sizeof(int64_t));
    c->slice_base[0] = 0;
    for (unsigned a = 0; a < c->td; ++a) c->slice_base[a + 1] = c->slice_base[a] + c->widths[a];
    c->total_bins = c->slice_base[c->td];
}

/* Per-slice projection constants, RangeLib.h:1007-1061. */
static void cddt_slice_constants(orc_cddt* c) {
    unsigned td = c->td;
    c->widths = (int*)malloc(td * sizeof(int));
    c->trans = (float*)malloc(td * sizeof(float));
    for (unsigned i = 0; i < td; ++i) {
        float angle = (float)(int)i * c->twopi_div_td;
        float rotated_height = fabsf((float)c->width * sinf(angle)) + fabsf((float)c->height * cosf(angle));
        c->widths[i] = (int)(unsigned)ceil((double)rotated_height - ORC_EPSILON);
        float left_top = (float)c->height * cosf(angle);
        float right_top = (float)c->width * sinf(angle) + (float)c->height * cosf(angle);
        float right_bottom = (float)c->width * sinf(angle);
        float min_y = ref_minf(left_top, ref_minf(right_top, right_bottom));
        double tr = -1.0 * (double)min_y - ORC_EPSILON;
        c->trans[i] = (float)((0.0 < tr) ? tr : 0.0);
    }
}

orc_cddt* orc_cddt_build(const uint8_t* occ, int width, int height, float max_range, unsigned td) {
    orc_cddt* c = (orc_cddt*)calloc(1, sizeof(orc_cddt));
    c->width = width; c->height = height; c->occ = occ; c->max_range = max_range; c->td = td;
    c->td_div_2pi = (float)((double)td / ORC_M_2PI);
    c->twopi_div_td = (float)(ORC_M_2PI / (double)(float)td);
    cddt_slice_constants(c);
    cddt_alloc_slices(c);

    size_t N = (size_t)width * height;
    uint8_t* edge = (uint8_t*)malloc(N ? N : 1);
    orc_edge_map(occ, width, height, edge);

    int64_t nb = c->total_bins;
    int64_t* count = (int64_t*)calloc((size_t)nb + 1, sizeof(int64_t));
    unsigned nslices = 0;
    while ((double)nslices < td / 2.0) ++nslices;       /* for (a = 0; a < td / 2.0; ++a) */
    if (nslices > td) nslices = td;

    /* two passes over the edge pixels: count, then fill (RangeLib.h:1083-1129) */
    for (int pass = 0; pass < 2; ++pass) {
        int64_t* cursor = NULL;
        if (pass == 1) {
            c->bin_start = (int64_t*)malloc(((size_t)nb + 1) * sizeof(int64_t));
            c->bin_start[0] = 0;
            for (int64_t b = 0; b < nb; ++b) c->bin_start[b + 1] = c->bin_start[b] + count[b];
            c->zeros = (float*)malloc((size_t)(c->bin_start[nb] ? c->bin_start[nb] : 1) * sizeof(float));
            cursor = (int64_t*)malloc(((size_t)nb + 1) * sizeof(int64_t));
            memcpy(cursor, c->bin_start, (size_t)nb * sizeof(int64_t));
        }
        for (int x = 0; x < width; ++x)
            for (int y = 0; y < height; ++y) {
                if (!edge[(size_t)x * height + y]) continue;
                float pcx = (float)(x + 0.5), pcy = (float)(y + 0.5);
                for (unsigned a = 0; a < nslices; ++a) {
                    float angle = (float)(int)a * c->twopi_div_td;
                    float ca = cosf(angle), sa = sinf(angle);
                    float half = (float)((double)(fabsf(sa) + fabsf(ca)) / 2.0);
                    float lcx = pcx * ca - pcy * sa;
                    float lcy = (pcx * sa + pcy * ca) + c->trans[a];
                    int upper = (int)((double)(lcy + half) - ORC_EPSILON);
                    int lower = (int)((double)(lcy - half) + ORC_EPSILON);
                    for (int i = lower; i <= upper; ++i) {
                        if (i < 0 || i >= c->widths[a]) continue;   /* outside the slice: UB in the reference */
                        int64_t b = c->slice_base[a] + i;
                        if (pass == 0) count[b]++;
                        else c->zeros[cursor[b]++] = lcx;
                    }
                }
            }
        free(cursor);
    }
    free(count);
    free(edge);

    /* sort + unique each bin (RangeLib.h:1131-1142), then compact */
    int64_t w = 0;
    for (int64_t b = 0; b < nb; ++b) {
        int64_t lo = c->bin_start[b], hi = c->bin_start[b + 1];
        float* p = c->zeros + lo;
        int64_t len = hi - lo;
        if (len > 1) qsort(p, (size_t)len, sizeof(float), cmp_float);
        c->bin_start[b] = w;
        for (int64_t i = 0; i < len; ++i) {
            if (i > 0 && p[i] == p[i - 1]) continue;
            c->zeros[w++] = p[i];
        }
    }
    c->bin_start[nb] = w;
    return c;
}

int64_t orc_cddt_num_zeros(const orc_cddt* c) { return c->bin_start[c->total_bins]; }

void orc_cddt_free(orc_cddt* c) {
    if (!c) return;
    free(c->widths); free(c->trans); free(c->slice_base); free(c->bin_start); free(c->zeros);
    free(c);
}

int orc_cddt_load(orc_cddt* c, const int* widths, const float* trans,
                  const int64_t* bin_len, const float* zeros, int64_t nzeros) {
    for (unsigned a = 0; a < c->td; ++a)
        if (widths[a] != c->widths[a]) return -1;
    memcpy(c->trans, trans, c->td * sizeof(float));
    int64_t nb = c->total_bins;
    c->bin_start[0] = 0;
    for (int64_t b = 0; b < nb; ++b) c->bin_start[b + 1] = c->bin_start[b] + bin_len[b];
    if (c->bin_start[nb] != nzeros) return -2;
    free(c->zeros);
    c->zeros = (float*)malloc((size_t)(nzeros ? nzeros : 1) * sizeof(float));
    memcpy(c->zeros, zeros, (size_t)nzeros * sizeof(float));
    return 0;
}

/* RangeLib.h:1287-1340 (_USE_ALTERNATE_MOD, _USE_CACHED_CONSTANTS, roundf). */
void orc_cddt_discretize(const orc_cddt* c, float theta, int* binned, float* discrete, int* flipped) {
    int it = 0;
    if (theta < 0.0) {
        while (theta < 0.0 && it++ < ORC_MAX_WRAP) theta = (float)((double)theta + ORC_M_2PI);
    } else if (theta > ORC_M_2PI) {
        while (theta > ORC_M_2PI && it++ < ORC_MAX_WRAP) theta = (float)((double)theta - ORC_M_2PI);
    }
    int fl = 0;
    if (theta >= ORC_M_PI) {
        fl = 1;
        theta = (float)((double)theta - ORC_M_PI);
    }
    int rounded = f2i(roundf(theta * c->td_div_2pi));
    if ((unsigned)rounded == (c->td >> 1)) {
        rounded = 0;
        fl = !fl;
    }
    int b = (int)((unsigned)rounded % c->td);
    *binned = b;
    *discrete = (float)b * c->twopi_div_td;
    *flipped = fl;
}

static inline int cddt_occupied(const orc_cddt* c, float x, float y) {
    /* map.grid[x][y] with float indices (RangeLib.h:1413, 1475) */
    if (!(x > -1.0f) || !(y > -1.0f)) return 0;
    if (x >= (float)c->width || y >= (float)c->height) return 0;
    size_t xi = (size_t)x, yi = (size_t)y;
    return c->occ[xi * c->height + yi] != 0;
}

float orc_cddt_calc_range(const orc_cddt* c, float x, float y, float heading, int* probes) {
    int a, fl;
    float dtheta;
    if (probes) *probes = -1;
    if (x != x || y != y || heading != heading) return c->max_range;
    orc_cddt_discretize(c, (float)(-1.0 * (double)heading), &a, &dtheta, &fl);
    float ca = cosf(dtheta), sa = sinf(dtheta);
    float lx = x * ca - y * sa;
    float ly = (x * sa + y * ca) + c->trans[a];
    unsigned li = (unsigned)f2i(ly);
    if (li >= (unsigned)c->widths[a]) return c->max_range;
    int64_t b = c->slice_base[a] + li;
    const float* bin = c->zeros + c->bin_start[b];
    int n = (int)(c->bin_start[b + 1] - c->bin_start[b]);
    if (probes) *probes = n;
    int high = n - 1;
    if (fl) {
        if (high == -1) return c->max_range;
        if (bin[0] > lx) return c->max_range;
        if (bin[high] < lx) return lx - bin[high];
        if (cddt_occupied(c, x, y)) return 0.0f;
        if (high > ORC_BSEARCH_THRESHOLD) {
            int lo = 0, hi = n;                         /* upper_bound */
            while (lo < hi) { int mid = (lo + hi) >> 1; if (lx < bin[mid]) hi = mid; else lo = mid + 1; }
            return lx - bin[lo - 1];
        }
        for (int i = high; i >= 0; --i)
            if (bin[i] <= lx) return lx - bin[i];
    } else {
        if (high == -1) return c->max_range;
        if (bin[high] < lx) return c->max_range;
        if (bin[0] > lx) return bin[0] - lx;
        if (cddt_occupied(c, x, y)) return 0.0f;
        if (high > ORC_BSEARCH_THRESHOLD) {
            int lo = 0, hi = n;                         /* upper_bound */
            while (lo < hi) { int mid = (lo + hi) >> 1; if (lx < bin[mid]) hi = mid; else lo = mid + 1; }
            if (lo == n) return 0.0f;                   /* x == last zero point: UB read in the reference */
            return bin[lo] - lx;
        }
        for (int i = 0; i < n; ++i)
            if (bin[i] >= lx) return bin[i] - lx;
    }
    return -1.0f;
}

/* prune, RangeLib.h:1176-1283.
 *
 * In the linear-search branch (bins of <= 65 entries) the reference leaves
 * `index` unassigned when no zero point is >= x (RangeLib.h:1242-1247: the
 * free cell lies more than max_range beyond the bin's last zero point).  The
 * compiled reference then reuses the value `index` last received, so it
 * marks that stale index (and the one before it) in the current bin; the
 * golden tables reproduce exactly under that reading.  This restatement
 * carries the last assigned index through the cells of a slice in the
 * reference's visiting order (x outer, y inner), starting each slice at 0. */
typedef struct { orc_cddt* c; float mr; uint8_t* used; } prune_ctx;

static void prune_slices(void* p, int lo, int hi) {
    prune_ctx* ctx = (prune_ctx*)p;
    orc_cddt* c = ctx->c;
    for (int a = lo; a < hi; ++a) {
        float angle = (float)a * c->twopi_div_td;
        float ca = cosf(angle), sa = sinf(angle);
        float tr = c->trans[a];
        int index = 0;   /* the reference's `index`, carried across cells */
        for (int x = 0; x < c->width; ++x) {
            float fx = (float)(0.5 + x);
            for (int y = 0; y < c->height; ++y) {
                float fy = (float)(0.5 + y);
                float lx = fx * ca - fy * sa;
                float ly = (fx * sa + fy * ca) + tr;
                unsigned li = (unsigned)f2i(ly);
                if (li >= (unsigned)c->widths[a]) continue;   /* unchecked in the reference */
                int64_t b = c->slice_base[a] + li;
                int64_t base = c->bin_start[b];
                const float* bin = c->zeros + base;
                int n = (int)(c->bin_start[b + 1] - base);
                int high = n - 1;
                if (high == -1) continue;
                if (c->occ[(size_t)x * c->height + y]) continue;
                if (bin[high] < lx && lx - bin[high] < ctx->mr) { ctx->used[base + high] = 1; continue; }
                if (high > ORC_BSEARCH_THRESHOLD) {
                    int l = 0, h = n;                            /* lower_bound */
                    while (l < h) { int mid = (l + h) >> 1; if (bin[mid] < lx) l = mid + 1; else h = mid; }
                    index = l;
                } else {
                    for (int i = 0; i < n; ++i) if (bin[i] >= lx) { index = i; break; }
                }
                if (index >= 0 && index < n) ctx->used[base + index] = 1;
                if (index - 1 >= 0 && index - 1 < n) ctx->used[base + index - 1] = 1;
            }
        }
    }
}

void orc_cddt_prune(orc_cddt* c, float max_range) {
    int64_t nz = orc_cddt_num_zeros(c);
    uint8_t* used = (uint8_t*)calloc((size_t)(nz ? nz : 1), 1);
    int nslices = 0;
    while ((double)nslices < c->td / 2.0) ++nslices;
    if (nslices > (int)c->td) nslices = (int)c->td;
    prune_ctx ctx = {c, max_range, used};
    orc_parallel(prune_slices, &ctx, nslices, 8);
    int64_t w = 0, nb = c->total_bins;
    for (int64_t b = 0; b < nb; ++b) {
        int64_t lo = c->bin_start[b], hi = c->bin_start[b + 1];
        c->bin_start[b] = w;
        for (int64_t i = lo; i < hi; ++i) {
            /* only slices a < td/2 are pruned; later slices are kept as is (they are empty) */
            if (used[i] || b >= c->slice_base[nslices]) c->zeros[w++] = c->zeros[i];
        }
    }
    c->bin_start[nb] = w;
    free(used);
}

/* ------------------------------------------------------------------ */
/* RangeMethod batched wrappers, RangeLib.h:439-612                      */
/* ------------------------------------------------------------------ */
/* calc_range_pair, RangeLib.h:1521-1615.  The reference indexes the bin with an unchecked
 * (int) lut_space_y; here a bin outside the slice gives (max_range, max_range).  Its forward
 * branch tests the occupancy without returning (RangeLib.h:1580), which is kept: the search
 * goes on. */
void orc_cddt_calc_range_pair(const orc_cddt* c, float x, float y, float heading, float* r, float* r_inv) {
    const float mr = c->max_range;
    int a, fl;
    float dtheta;
    *r = mr;
    *r_inv = mr;
    if (x != x || y != y || heading != heading) return;
    orc_cddt_discretize(c, (float)(-1.0 * (double)heading), &a, &dtheta, &fl);
    float ca = cosf(dtheta), sa = sinf(dtheta);
    float lx = x * ca - y * sa;
    float ly = (x * sa + y * ca) + c->trans[a];
    unsigned li = (unsigned)f2i(ly);
    if (li >= (unsigned)c->widths[a]) return;
    int64_t b = c->slice_base[a] + li;
    const float* bin = c->zeros + c->bin_start[b];
    int n = (int)(c->bin_start[b + 1] - c->bin_start[b]);
    int high = n - 1;
    if (high == -1) return;
    if (fl) {
        if (bin[0] > lx) { float d = bin[0] - lx; *r_inv = d < mr ? d : mr; return; }
        if (bin[high] < lx) { *r = lx - bin[high]; return; }
        if (cddt_occupied(c, x, y)) { *r = 0.0f; *r_inv = 0.0f; return; }
        int idx = high;                                 /* last zero point <= lx */
        while (idx > 0 && bin[idx] > lx) --idx;
        *r = lx - bin[idx];
        if (idx + 1 != n) *r_inv = bin[idx + 1] - lx;
    } else {
        if (bin[high] < lx) { float d = lx - bin[high]; *r_inv = d < mr ? d : mr; return; }
        int idx = 0;                                    /* first zero point >= lx */
        while (idx < high && bin[idx] < lx) ++idx;
        *r = bin[idx] - lx;
        if (idx - 1 != -1) *r_inv = lx - bin[idx - 1];
    }
}

/* ---- GiantLUTCast, RangeLib.h:1772-1904 (cached constants, 16-bit entries) ---- */
typedef struct { orc_glt* g; const float* dt; } glt_ctx;

static void glt_rows(void* p, int lo, int hi) {
    glt_ctx* k = (glt_ctx*)p;
    orc_glt* g = k->g;
    for (int x = lo; x < hi; ++x)
        for (int y = 0; y < g->height; ++y)
            for (unsigned i = 0; i < g->td; ++i) {
                float angle = (float)i * g->twopi_div_td;
                float r = orc_rm_calc_range(k->dt, g->width, g->height, g->max_range, (float)x, (float)y, angle, NULL);
                r = r < g->max_range ? r : g->max_range;                  /* std::min(max_range, r) */
                g->lut[((size_t)x * g->height + y) * g->td + i] = (uint16_t)(r * g->limits_div_max);
            }
}

orc_glt* orc_glt_build(const float* dt, int width, int height, float max_range, unsigned td, int nthreads) {
    orc_glt* g = (orc_glt*)calloc(1, sizeof(orc_glt));
    g->width = width;
    g->height = height;
    g->td = td;
    g->max_range = max_range;
    g->td_div_2pi = (float)((double)td / ORC_M_2PI);
    g->twopi_div_td = (float)(ORC_M_2PI / (double)(float)td);
    g->max_div_limits = max_range / 65535;
    g->limits_div_max = 65535 / max_range;
    g->lut = (uint16_t*)malloc((size_t)width * height * td * sizeof(uint16_t) + 1);
    glt_ctx k = {g, dt};
    orc_parallel(glt_rows, &k, width, nthreads);
    return g;
}

void orc_glt_free(orc_glt* g) {
    if (!g) return;
    free(g->lut);
    free(g);
}

/* discretize_theta, RangeLib.h:1834-1867 (alternate mod, cached constants, roundf) */
int orc_glt_discretize(const orc_glt* g, float theta) {
    int it = 0;
    if (theta < 0.0) {
        while (theta < 0.0 && it++ < ORC_MAX_WRAP) theta = (float)((double)theta + ORC_M_2PI);
    } else if (theta > ORC_M_2PI) {
        while (theta > ORC_M_2PI && it++ < ORC_MAX_WRAP) theta = (float)((double)theta - ORC_M_2PI);
    }
    int rounded = f2i(roundf(theta * g->td_div_2pi));
    return (int)((unsigned)rounded % g->td);
}

float orc_glt_calc_range(const orc_glt* g, float x, float y, float heading) {
    if (x != x || y != y || heading != heading) return g->max_range;
    if (x < 0 || x >= (float)g->width || y < 0 || y >= (float)g->height) return g->max_range;
    int b = orc_glt_discretize(g, heading);
    return g->lut[((size_t)f2i(x) * g->height + f2i(y)) * g->td + b] * g->max_div_limits;
}

float orc_method_calc_range(const orc_method* m, float x, float y, float heading, int* steps) {
    switch (m->kind) {
    case ORC_BL: return orc_bl_calc_range(m->occ, m->width, m->height, m->max_range, x, y, heading, steps);
    case ORC_RM: return orc_rm_calc_range(m->dt, m->width, m->height, m->max_range, x, y, heading, steps);
    case ORC_GLT: if (steps) *steps = 1; return orc_glt_calc_range(m->glt, x, y, heading);
    default: return orc_cddt_calc_range(m->cddt, x, y, heading, steps);
    }
}

/* one ray of a batched call: the method's own cos/sin, or the per-ray override (BL and RM) */
static inline float ray_range(const orc_method* m, float x, float y, float heading, size_t ray) {
    if (m->trig && m->kind == ORC_RM)
        return orc_rm_calc_range_trig(m->dt, m->width, m->height, m->max_range, x, y, m->trig[2 * ray],
                                      m->trig[2 * ray + 1], NULL);
    if (m->trig && m->kind == ORC_BL)
        return orc_bl_calc_range_trig(m->occ, m->width, m->height, m->max_range, x, y, m->trig[2 * ray],
                                      m->trig[2 * ray + 1], NULL);
    return orc_method_calc_range(m, x, y, heading, NULL);
}

typedef struct { float inv_s, s, rc; } world_consts;

static world_consts make_world(const orc_world* w) {
    world_consts k;
    k.inv_s = (float)(1.0 / (double)w->scale);                         /* RangeLib.h:442 */
    k.s = w->scale;
    k.rc = (float)(-1.0 * (double)w->angle - 3.0 * ORC_M_PI / 2.0);    /* RangeLib.h:450 */
    return k;
}

/* world pose -> (first, second) argument of calc_range, RangeLib.h:468-475 */
static inline void world_to_grid(const orc_world* w, const world_consts* k, const float* in,
                                 float* ax, float* ay, float* th) {
    float x = (in[0] - w->origin_x) * k->inv_s;
    float y = (in[1] - w->origin_y) * k->inv_s;
    float tmp = x;
    x = w->cos_angle * x - w->sin_angle * y;
    y = w->sin_angle * tmp + w->cos_angle * y;
    *th = -in[2] + k->rc;
    *ax = y;    /* calc_range(y, x, theta) */
    *ay = x;
}

typedef struct {
    const orc_method* m; const float* ins; const float* angles; const float* obs;
    float* outs; double* wouts; const float* ranges; int na; world_consts k;
} batch_ctx;

static void numpy_range_body(void* p, int lo, int hi) {
    batch_ctx* b = (batch_ctx*)p;
    for (int i = lo; i < hi; ++i) {
        float ax, ay, th;
        world_to_grid(&b->m->world, &b->k, b->ins + 3 * (size_t)i, &ax, &ay, &th);
        b->outs[i] = ray_range(b->m, ax, ay, th, (size_t)i) * b->k.s;
    }
}

void orc_numpy_calc_range(const orc_method* m, const float* ins, float* outs, int n, int nthreads) {
    batch_ctx b = {m, ins, NULL, NULL, outs, NULL, NULL, 0, make_world(&m->world)};
    orc_parallel(numpy_range_body, &b, n, nthreads);
}

/* calc_range_many_radial_optimized, RangeLib.h:616-676.  The reference writes in this order
 * per particle: for a = 0..P (P = num_rays / 3.0): row[a] = r(a), row[a + K] = r_inv(a);
 * then row[a] = calc_range(a) for a = P+1..K-1, with K = roundf((num_rays - 1) * pi /
 * (max - min)) and the heading offset accumulated as angle += step.  It is restated
 * literally, with writes outside the row dropped. */
void orc_cddt_radial(const orc_method* m, const float* ins, float* outs, int n, int num_rays,
                     float min_angle, float max_angle) {
    world_consts k = make_world(&m->world);
    float step = (max_angle - min_angle) / (float)(num_rays - 1);
    int max_pair = (int)((double)(float)num_rays / 3.0);
    float off_f = (float)(((double)num_rays - 1.0) * ORC_M_PI / (double)(max_angle - min_angle));
    int off = f2i(roundf(off_f));
    for (int i = 0; i < n; ++i) {
        float ax, ay, th;
        world_to_grid(&m->world, &k, ins + 3 * (size_t)i, &ax, &ay, &th);
        float* row = outs + (size_t)i * num_rays;
        float angle = min_angle;
        for (int a = 0; a <= max_pair; ++a) {
            float r, ri;
            orc_cddt_calc_range_pair(m->cddt, ax, ay, th - angle, &r, &ri);
            if (a >= 0 && a < num_rays) row[a] = r * k.s;
            if (a + off >= 0 && a + off < num_rays) row[a + off] = ri * k.s;
            angle += step;
        }
        for (int a = max_pair + 1; a < off; ++a) {
            if (a < num_rays) row[a] = orc_cddt_calc_range(m->cddt, ax, ay, th - angle, NULL) * k.s;
            angle += step;
        }
    }
}

static void raw_range_body(void* p, int lo, int hi) {
    batch_ctx* b = (batch_ctx*)p;
    for (int i = lo; i < hi; ++i) {
        const float* q = b->ins + 3 * (size_t)i;
        b->outs[i] = ray_range(b->m, q[0], q[1], q[2], (size_t)i);
    }
}

void orc_calc_range_many_raw(const orc_method* m, const float* ins, float* outs, int n, int nthreads) {
    batch_ctx b = {m, ins, NULL, NULL, outs, NULL, NULL, 0, make_world(&m->world)};
    orc_parallel(raw_range_body, &b, n, nthreads);
}

static void angles_body(void* p, int lo, int hi) {
    batch_ctx* b = (batch_ctx*)p;
    for (int i = lo; i < hi; ++i) {
        float ax, ay, th;
        world_to_grid(&b->m->world, &b->k, b->ins + 3 * (size_t)i, &ax, &ay, &th);
        for (int a = 0; a < b->na; ++a)
            b->outs[(size_t)i * b->na + a] = ray_range(b->m, ax, ay, th - b->angles[a], (size_t)i * b->na + a) * b->k.s;
    }
}

void orc_numpy_calc_range_angles(const orc_method* m, const float* ins, const float* angles,
                                 float* outs, int n, int na, int nthreads) {
    batch_ctx b = {m, ins, angles, NULL, outs, NULL, NULL, na, make_world(&m->world)};
    orc_parallel(angles_body, &b, n, nthreads);
}

static inline int sensor_bin(float v, int K) {
    /* std::min<float>(std::max<float>(v, 0.0), (float)K - 1.0) then (int) */
    float hi = (float)((double)(float)K - 1.0);
    v = ref_minf(ref_maxf(v, 0.0f), hi);
    if (v != v) return 0;
    return (int)v;
}

static void eval_body(void* p, int lo, int hi) {
    batch_ctx* b = (batch_ctx*)p;
    const orc_method* m = b->m;
    int K = m->K;
    for (int i = lo; i < hi; ++i) {
        double weight = 1.0;
        for (int j = 0; j < b->na; ++j) {
            int r = sensor_bin(b->obs[j] * b->k.inv_s, K);
            int d = sensor_bin(b->ranges[(size_t)i * b->na + j] * b->k.inv_s, K);
            weight *= m->table[(size_t)r * K + d];
        }
        b->wouts[i] = weight;
    }
}

/* RangeLib.h:533-555 */
void orc_eval_sensor_model(const orc_method* m, const float* obs, const float* ranges,
                           double* outs, int rays_per_particle, int particles, int nthreads) {
    batch_ctx b = {m, NULL, NULL, obs, NULL, outs, ranges, rays_per_particle, make_world(&m->world)};
    orc_parallel(eval_body, &b, particles, nthreads);
}

static void fused_body(void* p, int lo, int hi) {
    batch_ctx* b = (batch_ctx*)p;
    const orc_method* m = b->m;
    int K = m->K;
    for (int i = lo; i < hi; ++i) {
        float ax, ay, th;
        world_to_grid(&m->world, &b->k, b->ins + 3 * (size_t)i, &ax, &ay, &th);
        double weight = 1.0;
        for (int a = 0; a < b->na; ++a) {
            float d = ray_range(m, ax, ay, th - b->angles[a], (size_t)i * b->na + a);
            int di = sensor_bin(d, K);
            int ri = sensor_bin(b->obs[a] * b->k.inv_s, K);
            weight *= m->table[(size_t)ri * K + di];
        }
        b->wouts[i] = weight;
    }
}

/* RangeLib.h:558-612: ranges stay in pixels (no world-scale round trip) */
void orc_calc_range_repeat_angles_eval_sensor_model(const orc_method* m, const float* ins,
                                                    const float* angles, const float* obs,
                                                    double* weights, int n, int na, int nthreads) {
    batch_ctx b = {m, ins, angles, obs, NULL, weights, NULL, na, make_world(&m->world)};
    orc_parallel(fused_body, &b, n, nthreads);
}

void orc_world_rays(const orc_world* w, const float* ins, const float* angles, int n, int na,
                    float* xyh, float* trig) {
    world_consts k = make_world(w);
    int per = angles ? na : 1;
    for (int i = 0; i < n; ++i) {
        float ax, ay, th;
        world_to_grid(w, &k, ins + 3 * (size_t)i, &ax, &ay, &th);
        for (int a = 0; a < per; ++a) {
            float h = angles ? th - angles[a] : th;
            size_t r = (size_t)i * per + a;
            if (xyh) { xyh[3 * r] = ax; xyh[3 * r + 1] = ay; xyh[3 * r + 2] = h; }
            if (trig) { trig[2 * r] = cosf(h); trig[2 * r + 1] = sinf(h); }
        }
    }
}

double orc_mean_steps(const orc_method* m, const float* ins, const float* angles, int n, int na) {
    world_consts k = make_world(&m->world);
    int per = angles ? na : 1;
    double total = 0.0;
    for (int i = 0; i < n; ++i) {
        float ax, ay, th;
        world_to_grid(&m->world, &k, ins + 3 * (size_t)i, &ax, &ay, &th);
        for (int a = 0; a < per; ++a) {
            int s = 0;
            orc_method_calc_range(m, ax, ay, angles ? th - angles[a] : th, &s);
            total += s;
        }
    }
    return (n > 0 && per > 0) ? total / ((double)n * per) : 0.0;
}
