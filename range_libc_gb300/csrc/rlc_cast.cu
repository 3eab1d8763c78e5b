// Ray casting kernels: Bresenham's line, ray marching on the distance
// transform and CDDT queries, the world-frame batched wrappers, the sensor
// model and the fused cast + sensor-model particle update.
//
// Every parity-relevant float operation is an explicit round-to-nearest
// intrinsic (__fmul_rn, __fadd_rn, ...) so that no multiply-add is ever
// contracted into an FMA: the reference is plain IEEE float/double C++
// (RangeLib.h), and its results are reproduced bit for bit.  Mixed
// float/double expressions of the reference are evaluated in double here
// too, except where the float evaluation is provably identical (noted).
// The only source of difference is the per-ray cosf/sinf of RM and BL: here
// they are the correctly rounded values (rlc_trig.cuh), which a host libm
// matches on all but ~0.1 % of arguments (glibc's float sine and cosine are
// not correctly rounded); the optional per-ray trig override takes the
// host's values instead, for parity tests.
#include "rlc_internal.cuh"

#include <climits>

namespace rlc {
namespace {

constexpr double kM2Pi = 6.28318530718;           // RangeLib.h:61 M_2PI
constexpr double kMPi = 3.14159265358979323846;   // <cmath> M_PI
constexpr int kBinarySearchThreshold = 64;         // RangeLib.h:62
constexpr int kMaxWrap = 100000;                   // bound on discretize_theta's loops
// For a float t, (double)t > M_2PI <=> t > kM2PiDownF (the largest float below
// M_2PI) and (double)t >= M_PI <=> t >= kMPiUpF (the smallest float above
// M_PI): the range tests of discretize_theta stay off the FP64 pipe.
constexpr float kM2PiDownF = 0x1.921fb4p+2f;
constexpr float kMPiUpF = 0x1.921fb6p+1f;
// (float)((double)t - M_PI) for every float t in [kMPiUpF, kM2PiDownF] equals
// (t - kMPiHiF) - kMPiLoF in float arithmetic: the first difference is exact
// (Sterbenz) and the second rounds like the double expression -- checked for
// all 8,388,608 floats of the interval (tests/test_float_identities.py).
constexpr float kMPiHiF = 0x1.921fb6p+1f;     // (float)M_PI
constexpr float kMPiLoF = -0x1.777a5cp-24f;   // (float)(M_PI - kMPiHiF)
constexpr int kPrefetch = 8;                        // RM prefetch distance (px) of the prefetching schedule
constexpr int kAnyKind = -1;                        // k_batch: kind, layout and prefetch chosen per filter
constexpr int kRmOnly = -2;                         // k_batch: every filter ray-marches (LAYOUT, PF given)

__device__ __forceinline__ float ref_maxf(float a, float b) { return (a < b) ? b : a; }

// r / d for 0 <= r < 2^24 and d >= 1, given inv_d = 1 / (float)d rounded to nearest: the float
// quotient is within one of the true one, and one remainder test corrects it
__device__ __forceinline__ int div_small(int r, int d, float inv_d) {
    int q = __float2int_rz(__fmul_rn(__int2float_rn(r), inv_d));
    const int rem = r - q * d;
    return q + (rem >= d) - (rem < 0);
}
__device__ __forceinline__ float ref_minf(float a, float b) { return (b < a) ? b : a; }

// ---------------------------------------------------------------- map access
__device__ __forceinline__ size_t u16_index(const MapDev& m, int x, int y) {
    return ((((size_t)(x >> 3) * m.tiles_y + (y >> 3))) << 6) + ((((x >> 2) & 1) << 1 | ((y >> 2) & 1)) << 4) +
           (((x & 3) << 2) | (y & 3));
}

template <int LAYOUT>
__device__ __forceinline__ float dt_at(const MapDev& m, int x, int y) {
    if (LAYOUT == DT_U16) {
        const unsigned v = __ldg(m.dt16 + u16_index(m, x, y));
        if (v == 0xFFFFu) return __ldg(m.dt + (size_t)x * m.H + y);   // d^2 >= 65535: the float itself
        return __fsqrt_rn(__uint2float_rn(v));                         // == sqrtf(D) of the distance transform
    }
    if (LAYOUT == DT_TILED)
        return __ldg(m.dt + (((size_t)(x >> 3) * m.tiles_y + (y >> 3)) << 6) + ((x & 7) << 3) + (y & 7));
    if (LAYOUT == DT_STEP || LAYOUT == DT_RUNS) return __ldg(m.step + (size_t)x * m.H + y);   // the step (0 on walls)
    return __ldg(m.dt + (size_t)x * m.H + y);
}

template <int LAYOUT>
__device__ __forceinline__ const void* dt_ptr(const MapDev& m, int x, int y) {
    if (LAYOUT == DT_U16) return m.dt16 + u16_index(m, x, y);
    if (LAYOUT == DT_TILED)
        return m.dt + (((size_t)(x >> 3) * m.tiles_y + (y >> 3)) << 6) + ((x & 7) << 3) + (y & 7);
    if (LAYOUT == DT_STEP || LAYOUT == DT_RUNS) return m.step + (size_t)x * m.H + y;
    return m.dt + (size_t)x * m.H + y;
}

__device__ __forceinline__ void prefetch_l1(const void* p) {
    asm volatile("prefetch.global.L1 [%0];" ::"l"(p));
}

__device__ __forceinline__ bool occ_at(const MapDev& m, int x, int y) {
    if ((unsigned)x >= (unsigned)m.W || (unsigned)y >= (unsigned)m.H) return false;
    uint64_t w = __ldg(m.bits + (size_t)(x >> 3) * m.tiles_y + (y >> 3));
    return (w >> (((x & 7) << 3) | (y & 7))) & 1ull;
}

// ------------------------------------------------------- ray marching (RM)
// RangeLib.h:927-962 (RayMarching::calc_range).  t grows by >= 1 per step,
// so the loop runs at most ceil(max_range) + 1 times.
//
// PF > 0: every step also issues an L1 prefetch of the cell PF pixels
// further along the ray.  Near walls the march advances ~1 px per step, so
// the cell a later step reads is already on its way when that step starts;
// the prefetch is a hint and never changes a result.
//
// DT_RUNS: the step map plus equal-step runs (run_skip below).
constexpr int kMinRun = 12;       // shortest run worth a skip
constexpr int kRunTrigger = 6;    // equal steps in a row before the run map is read

// Exact skip over a run of equal steps (DT_RUNS).  A ray running beside a wall keeps the same
// distance to it, so its march repeats one step value v for many iterations: the longest rays of
// a particle-filter step repeat a step of 1 (one pixel) or 1.998 over a hundred times.  Once a
// ray has taken kRunTrigger equal steps in a row, at cell (px, py), the run map says how many
// cells after it along the ray's major axis (L, direction of travel) have step v too (only then:
// the read would lengthen the march of every other ray).  The march parameters of such a
// run are known without reading a cell: t_j+1 = t_j + v rounded as the reference's addition.  An
// estimate J of how many positions t_1 .. t_J stay in the box {the current row or column} x {the
// run} is checked exactly at t_J with the march's own float operations; positions are monotone in
// t, so every position before t_J lies in the box too -- a cell of step v in the grid -- and
// t_J+1 < max_range keeps the reference's loop going.  The march then resumes at t_J+1 having
// counted J steps, exactly where the reference's loop is after J more iterations.  Returns t1 (the
// parameter after the current step) when no skip applies.
__device__ __forceinline__ float run_skip(float mr, float x0, float y0, float c, float s, int px, int py, int L, float v,
                                       float t1, int* steps) {
    const bool ydom = fabsf(s) >= fabsf(c);
    const float dmaj = ydom ? s : c, dmin = ydom ? c : s;
    const float o_maj = ydom ? y0 : x0, o_min = ydom ? x0 : y0;
    const int cmaj = ydom ? py : px, cmin = ydom ? px : py;
    // estimated parameter limits (the exact check below decides)
    float lim = (dmaj > 0.0f ? (float)(cmaj + L + 1) - o_maj : (float)(cmaj - L) - o_maj) / dmaj;
    if (dmin > 0.0f) lim = fminf(lim, ((float)(cmin + 1) - o_min) / dmin);
    else if (dmin < 0.0f) lim = fminf(lim, ((float)cmin - o_min) / dmin);
    lim = fminf(lim, mr - v);
    int J = (int)fminf((lim - t1) / v - 1.0f, 255.0f);
    for (int attempt = 0; attempt < 3 && J >= 2; ++attempt, J >>= 1) {
        float tj = t1;
        for (int j = 1; j < J; ++j) tj = __fadd_rn(tj, v);
        const int qx = __float2int_rz(__fadd_rn(x0, __fmul_rn(c, tj)));
        const int qy = __float2int_rz(__fadd_rn(y0, __fmul_rn(s, tj)));
        const int qmaj = ydom ? qy : qx, qmin = ydom ? qx : qy;
        const bool in_run = dmaj > 0.0f ? (qmaj >= cmaj && qmaj <= cmaj + L) : (qmaj <= cmaj && qmaj >= cmaj - L);
        const float tn = __fadd_rn(tj, v);
        if (qmin == cmin && in_run && tn < mr) {
            if (steps) *steps += J;
            return tn;
        }
    }
    return t1;
}

// A ray's march state (RangeLib.h:927-962): origin, direction, the parameter t, and for DT_RUNS
// the last step and how many equal steps in a row ended with it; r is the caller's ray index.
struct __align__(16) RmRay {
    float x0, y0, c, s, t, prev;
    int rep, r;
};

// Marches q from its parameter q.t.  BUDGETED: at most `budget` rounds of the loop (a run skip is
// one round), after which it returns false with q holding the state of the next round, exactly
// where the reference's loop stands; otherwise (and when the ray ends first) it returns true with
// the range in *out.  One exit test per step: an off-grid position reads cell (0, 0) and leaves.
template <int LAYOUT, int PF, bool BUDGETED>
__device__ __forceinline__ bool rm_advance(const MapDev& m, float mr, RmRay& q, int budget, float* out, int* steps) {
    const float x0 = q.x0, y0 = q.y0, c = q.c, s = q.s;
    float t = q.t, prev = q.prev;
    int rep = q.rep;   // equal steps in a row
    // DT_RUNS: the byte of the run word that lies along the ray (major axis, direction of travel)
    const unsigned run_shift = fabsf(s) >= fabsf(c) ? (s > 0.0f ? 0u : 8u) : (c > 0.0f ? 16u : 24u);
    for (int round = 0;; ++round) {
        if (BUDGETED && round >= budget) {
            q.t = t;
            q.prev = prev;
            q.rep = rep;
            return false;
        }
        const int px = __float2int_rz(__fadd_rn(x0, __fmul_rn(c, t)));
        const int py = __float2int_rz(__fadd_rn(y0, __fmul_rn(s, t)));
        const bool out_of_grid = (unsigned)px >= (unsigned)m.W || (unsigned)py >= (unsigned)m.H;
        if (PF > 0) {
            const float tp = t + (float)PF;
            const int qx = __float2int_rz(x0 + c * tp), qy = __float2int_rz(y0 + s * tp);
            if ((unsigned)qx < (unsigned)m.W && (unsigned)qy < (unsigned)m.H) prefetch_l1(dt_ptr<LAYOUT>(m, qx, qy));
        }
        // DT_STEP reads the step max(d * 0.999, 1) precomputed per cell (0 where d = 0).  The
        // linear layouts form the cell index in 32 bits (W * H < 2^31) and select it once.
        constexpr bool kStepMap = LAYOUT == DT_STEP || LAYOUT == DT_RUNS;
        float d;
        unsigned cell = 0u;
        if (LAYOUT == DT_LINEAR || kStepMap) {
            cell = out_of_grid ? 0u : (unsigned)px * (unsigned)m.H + (unsigned)py;
            d = __ldg((kStepMap ? m.step : m.dt) + cell);
        } else {
            d = dt_at<LAYOUT>(m, out_of_grid ? 0 : px, out_of_grid ? 0 : py);
        }
        if (steps && !out_of_grid) ++*steps;
        const float st = kStepMap ? d : ref_maxf(__fmul_rn(d, 0.999f), 1.0f);
        const float tn = __fadd_rn(t, st);
        const bool hit = d <= 0.0f;
        if (out_of_grid | hit | !(tn < mr)) {
            if (out_of_grid || !hit) {
                *out = mr;
            } else {
                const float xd = __fsub_rn(__int2float_rn(px), x0);
                const float yd = __fsub_rn(__int2float_rn(py), y0);
                *out = __fsqrt_rn(__fadd_rn(__fmul_rn(xd, xd), __fmul_rn(yd, yd)));
            }
            return true;
        }
        t = tn;
        if (LAYOUT == DT_RUNS) {
            rep = st == prev ? rep + 1 : 0;
            prev = st;
            if (rep == kRunTrigger) {   // a ray repeating one step (beside a wall): look for the run
                rep = 0;
                const int L = (int)((__ldg(m.runs + cell) >> run_shift) & 255u);
                if (L >= kMinRun) t = run_skip(mr, x0, y0, c, s, px, py, L, st, t, steps);
            }
        }
    }
}

// the march from t = 0; NaN arguments give max_range (the reference's loop never ends on them)
template <int LAYOUT, int PF = 0>
__device__ float rm_cast(const MapDev& m, float mr, float x0, float y0, float c, float s, int* steps = nullptr) {
    if (isnan(x0) || isnan(y0) || isnan(c) || isnan(s)) return mr;
    if (!(0.0f < mr)) return mr;
    RmRay q{x0, y0, c, s, 0.0f, -1.0f, 0, 0};
    float d = mr;
    rm_advance<LAYOUT, PF, false>(m, mr, q, 0, &d, steps);
    return d;
}

// ---------------------------------------------------- Bresenham's line (BL)
// RangeLib.h:696-769.  The occupancy word of the current 8x8 tile stays in a
// register; a new word is read only when the line leaves the tile.
struct BitCache {   // x, y in the grid; maps hold at most 2^31 cells (rlc_map_create), so < 2^26 tiles
    unsigned tile = 0xFFFFFFFFu;
    uint64_t word = 0;
    __device__ __forceinline__ bool test(const MapDev& m, int x, int y) {
        const unsigned t = (unsigned)(x >> 3) * (unsigned)m.tiles_y + (unsigned)(y >> 3);
        if (t != tile) { tile = t; word = __ldg(m.bits + t); }
        return (word >> (((x & 7) << 3) | (y & 7))) & 1ull;
    }
};

__device__ float bl_cast(const MapDev& m, float mr, float x, float y, float c, float s, unsigned* err,
                         int* steps = nullptr) {
    if (isnan(x) || isnan(y)) return mr;
    if (occ_at(m, __float2int_rz(x), __float2int_rz(y))) return 0.0f;
    if (isnan(c) || isnan(s)) return mr;   // the reference never terminates on a NaN heading
    float x0 = y, y0 = x;
    float x1 = __fadd_rn(y, __fmul_rn(mr, s));
    float y1 = __fadd_rn(x, __fmul_rn(mr, c));
    bool steep = fabsf(__fsub_rn(y1, y0)) > fabsf(__fsub_rn(x1, x0));
    if (steep) {
        float t = x0; x0 = y0; y0 = t;
        t = x1; x1 = y1; y1 = t;
    }
    const float deltax = fabsf(__fsub_rn(x1, x0));
    const float deltaerr = fabsf(__fsub_rn(y1, y0));
    float error = 0.0f;
    float _x = x0, _y = y0;
    const float xstep = (x0 < x1) ? 1.0f : -1.0f;
    const float ystep = (y0 < y1) ? 1.0f : -1.0f;
    const int end = __float2int_rz(__fadd_rn(x1, xstep));
    // the reference loop ends after at most |x1 - x0| + 3 steps unless the integer part of _x
    // never equals `end`: above 2^24 float +-1 no longer moves _x, and a start whose fraction is
    // 1 - ulp rounds up where the walk crosses a power of two (999.99994 + 24 -> 1025.0) and
    // skips that integer; the reference then never terminates, here the bound returns max_range
    const int bound = (int)(deltax < 1e9f ? deltax : 1e9f) + 4;
    // the reference's in-grid test is `0 <= g && g < (float)W`; (float)W rounds above 2^24, and the
    // floats below it are exactly the floats below min(W, (float)W) (none lies between W and a
    // (float)W rounded up)
    const unsigned bx = min((unsigned)m.W, __float2uint_rz(__int2float_rn(m.W)));
    const unsigned by = min((unsigned)m.H, __float2uint_rz(__int2float_rn(m.H)));
    // both walk coordinates move monotonically (_x by xstep, _y by ystep), so once a grid axis
    // has left [0, b) in its direction of motion no later cell is inside the grid: the walk
    // returns max_range there, as the reference's does when it ends (it walks on to its end cell)
    const bool gx_up = (steep ? xstep : ystep) > 0.0f, gy_up = (steep ? ystep : xstep) > 0.0f;
    int n = 0;
    BitCache cache;
    while (__float2int_rz(_x) != end) {
        if (n > bound) { atomicOr(err, F_BL_BOUND); return mr; }
        ++n;
        if (steps) ++*steps;
        _x = __fadd_rn(_x, xstep);
        error = __fadd_rn(error, deltaerr);
        // `error * 2.00 >= deltax` is a double comparison in the reference;
        // doubling a finite float is exact, so the float comparison is identical
        if (__fmul_rn(error, 2.0f) >= deltax) {
            _y = __fadd_rn(_y, ystep);
            error = __fsub_rn(error, deltax);
        }
        const float gx = steep ? _x : _y;   // isOccupied(_y, _x) when not steep
        const float gy = steep ? _y : _x;
        // `0 <= g && g < B` then (int)g: for an integer B, floor(g) < B exactly when g < B and
        // floor(g) >= 0 exactly when g >= 0 (-0.0 included; saturation keeps |g| >= 2^31 out),
        // and inside the grid floor equals truncation; g is never NaN here (NaN inputs end above)
        const int fx = __float2int_rd(gx), fy = __float2int_rd(gy);
        if ((unsigned)fx < bx && (unsigned)fy < by) {
            if (cache.test(m, fx, fy)) {
                float xd = __fsub_rn(_x, x0), yd = __fsub_rn(_y, y0);
                return __fsqrt_rn(__fadd_rn(__fmul_rn(xd, xd), __fmul_rn(yd, yd)));
            }
        } else if ((gx_up ? fx >= (int)bx : fx < 0) || (gy_up ? fy >= (int)by : fy < 0)) {
            return mr;   // past the grid's edge: no occupied cell is left on the walk
        }
    }
    return mr;
}

// ------------------------------------------------------------------ CDDT
// RangeLib.h:1287-1340 discretize_theta (alternate mod, cached constants)
__device__ __forceinline__ void cddt_discretize(const CddtDev& c, float theta, int& binned, bool& flipped,
                                                unsigned* err) {
    int it = 0;
    if (theta < 0.0f) {
        while (theta < 0.0f) {
            if (++it > kMaxWrap) { atomicOr(err, F_WRAP_BOUND); break; }
            theta = __double2float_rn(__dadd_rn((double)theta, kM2Pi));
        }
    } else if (theta > kM2PiDownF) {
        while (theta > kM2PiDownF) {
            if (++it > kMaxWrap) { atomicOr(err, F_WRAP_BOUND); break; }
            theta = __double2float_rn(__dsub_rn((double)theta, kM2Pi));
        }
    }
    bool fl = false;
    if (theta >= kMPiUpF) {
        fl = true;
        theta = theta <= kM2PiDownF ? __fsub_rn(__fsub_rn(theta, kMPiHiF), kMPiLoF)
                                    : __double2float_rn(__dsub_rn((double)theta, kMPi));   // after a bounded wrap
    }
    int rounded = __float2int_rz(roundf(__fmul_rn(theta, c.td_div_2pi)));
    if ((unsigned)rounded == (c.td >> 1)) {
        rounded = 0;
        fl = !fl;
    }
    binned = (int)((unsigned)rounded % c.td);
    flipped = fl;
}

// first index i of the sorted bin with bin[i] > v (upper) or bin[i] >= v (lower); n if none.
// bound_g: binary search.  bound_s (the sector schedule of CDDT methods) searches bins of more
// than kSectorSearch entries by whole sectors: each step reads the
// aligned 32-byte sector (8 zero points) around the midpoint with two 16-byte loads and settles
// every entry of it that lies in [lo, hi), so a bin of n entries takes about log2(n / 8) + 1
// dependent reads instead of log2(n), then finishes with the binary search.  It pays where the
// reads miss the L1 (queries spread over the map); where neighbouring queries share their bins'
// cache lines the plain search's fewer instructions win.  Zero-point arrays are allocated in whole sectors (cddt_zeros_bytes),
// so the sector reads stay inside the allocation; entries outside [lo, hi) are never used.
constexpr int kSectorSearch = 32;

__device__ __forceinline__ int bound_g(const float* __restrict__ bin, int n, float v, bool upper) {
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        const float z = __ldg(bin + mid);
        if (upper ? (v < z) : (v <= z)) hi = mid; else lo = mid + 1;
    }
    return lo;
}

// the aligned 32-byte sector around entry mid of a bin (two 16-byte reads)
struct Sector {
    float4 a, b;
};
__device__ __forceinline__ Sector sector_at(const float* __restrict__ bin, int mid) {
    const float4* sec = reinterpret_cast<const float4*>(reinterpret_cast<uintptr_t>(bin + mid) & ~(uintptr_t)31);
    return Sector{__ldg(sec), __ldg(sec + 1)};
}

// first: the sector of the first round (at n / 2), when the caller has already requested it
__device__ __forceinline__ int bound_s(const float* __restrict__ bin, int n, float v, bool upper,
                                      const Sector* first = nullptr) {
    int lo = 0, hi = n;
    bool pre = first != nullptr;
    while (hi - lo > kSectorSearch) {
        const int mid = (lo + hi) >> 1;
        const uintptr_t pm = reinterpret_cast<uintptr_t>(bin + mid);
        const int s0 = mid - (int)((pm & 31) >> 2);   // index in the bin of the sector's first entry
        const Sector sc = pre ? *first : sector_at(bin, mid);
        pre = false;
        const float4 a = sc.a, b = sc.b;
        const float z[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
        const int w0 = max(lo, s0), w1 = min(hi, s0 + 8);   // the sector's entries inside [lo, hi)
        int k = w1;                                          // first of them at or past the bound
#pragma unroll
        for (int j = 7; j >= 0; --j) {
            const int idx = s0 + j;
            if (idx >= w0 && idx < w1 && (upper ? (v < z[j]) : (v <= z[j]))) k = idx;
        }
        if (k == w1) lo = w1;                 // the whole window precedes the bound
        else if (k > w0) lo = hi = k;         // entry k - 1 precedes it and entry k does not
        else hi = w0;                         // the bound is at or before the window's start
    }
    return lo + bound_g(bin + lo, hi - lo, v, upper);
}

// The same bound computed by a whole warp for one query: 32 pivots per
// round, __ballot_sync narrows the range 32x, a last round scans <= 32
// consecutive zero points in one coalesced load.  All 32 lanes must call it
// with the same arguments.
__device__ __forceinline__ int bound_warp(const float* __restrict__ bin, int n, float v, bool upper) {
    const int lane = threadIdx.x & 31;
    const float inf = __int_as_float(0x7f800000);
    int lo = 0, hi = n;   // the answer lies in [lo, hi]
    while (hi - lo > 32) {
        const int step = (hi - lo + 31) >> 5;
        const int i = lo + lane * step;
        const float z = i < hi ? __ldg(bin + i) : inf;
        const unsigned m = __ballot_sync(0xffffffffu, upper ? (v < z) : (v <= z));
        const int f = m ? __ffs(m) - 1 : 32;
        const int nlo = f > 0 ? lo + (f - 1) * step + 1 : lo;
        const int nhi = f < 32 ? min(hi, lo + f * step) : hi;
        lo = nlo;
        hi = nhi;
    }
    const int i = lo + lane;
    const float z = i < hi ? __ldg(bin + i) : inf;
    const unsigned m = __ballot_sync(0xffffffffu, i < hi && (upper ? (v < z) : (v <= z)));
    return m ? lo + __ffs(m) - 1 : hi;
}

// A CDDT query up to its bin search (RangeLib.h:1342-1516).  Either the
// result is final (mode 0) or the bin search is pending:
//   mode 1  flipped:  the last zero point <= x (upper_bound - 1; the
//           reference's binary and linear branches agree on it)
//   mode 2  forward, bin > 65 entries: upper_bound (first > x)
//   mode 3  forward, bin <= 65 entries: the linear scan's first >= x
struct CddtPending {
    const float* bin;
    int n;
    float lx;
    int mode;
    Sector mid;   // SECTOR searches of bins longer than kSectorSearch: the first round's sector
};

// SECTOR: the sector search's first read (the sector at the bin's midpoint) is issued together with
// the bin's first and last entries instead of after them
template <bool SECTOR = false>
__device__ __forceinline__ float cddt_front(const CastParams& p, float x, float y, float heading, CddtPending& q) {
    const CddtDev& c = p.cddt;
    const float mr = p.mr;
    q.mode = 0;
    if (isnan(x) || isnan(y) || isnan(heading)) return mr;
    // grid[x][y] with float indices: the cell under the query point.  It depends on the pose alone,
    // so its read is issued first and overlaps the table reads below.
    const bool occ = (x > -1.0f) && (y > -1.0f) && occ_at(p.map, __float2int_rz(x), __float2int_rz(y));
    int a;
    bool fl;
    cddt_discretize(c, -heading, a, fl, p.err);   // discretize_theta(-1.0 * heading)
    const float ca = __ldg(c.cosv + a), sa = __ldg(c.sinv + a);
    const float lx = __fsub_rn(__fmul_rn(x, ca), __fmul_rn(y, sa));
    const float ly = __fadd_rn(__fadd_rn(__fmul_rn(x, sa), __fmul_rn(y, ca)), __ldg(c.trans + a));
    const unsigned li = (unsigned)__float2int_rz(ly);
    if (li >= (unsigned)__ldg(c.widths + a)) return mr;
    const unsigned b = __ldg(c.slice_base + a) + li;
    const unsigned lo = __ldg(c.bin_start + b);
    const int n = (int)(__ldg(c.bin_start + b + 1) - lo);
    const float* bin = c.zeros + lo;
    const int high = n - 1;
    if (high == -1) return mr;
    const float first = __ldg(bin), last = __ldg(bin + high);
    if (SECTOR && n > kSectorSearch) q.mid = sector_at(bin, n >> 1);
    q.bin = bin;
    q.n = n;
    q.lx = lx;
    if (fl) {
        if (first > lx) return mr;
        if (last < lx) return __fsub_rn(lx, last);
        if (occ) return 0.0f;
        q.mode = 1;
    } else {
        if (last < lx) return mr;
        if (first > lx) return __fsub_rn(first, lx);
        if (occ) return 0.0f;
        q.mode = high > kBinarySearchThreshold ? 2 : 3;
    }
    return 0.0f;
}

__device__ __forceinline__ float cddt_finish(const CastParams& p, const CddtPending& q, int idx) {
    if (q.mode == 1) return __fsub_rn(q.lx, __ldg(q.bin + idx - 1));
    if (idx == q.n) {   // x equals the last zero point: the reference reads past the bin
        atomicOr(p.err, F_CDDT_PAST_END);
        return 0.0f;
    }
    return __fsub_rn(__ldg(q.bin + idx), q.lx);
}

template <bool SECTOR = false>
__device__ float cddt_cast(const CastParams& p, float x, float y, float heading) {
    CddtPending q;
    const float r = cddt_front<SECTOR>(p, x, y, heading, q);
    if (q.mode == 0) return r;
    const bool upper = q.mode != 3;
    return cddt_finish(p, q, SECTOR ? bound_s(q.bin, q.n, q.lx, upper, q.n > kSectorSearch ? &q.mid : nullptr)
                                    : bound_g(q.bin, q.n, q.lx, upper));
}

// warp-cooperative variant: every lane resolves its own query up to the bin,
// then the warp searches the pending bins one query at a time
__device__ __forceinline__ float cddt_cast_warp(const CastParams& p, bool active, float x, float y, float heading) {
    CddtPending q;
    q.mode = 0;
    float r = active ? cddt_front(p, x, y, heading, q) : 0.0f;
    unsigned pending = __ballot_sync(0xffffffffu, q.mode != 0);
    int my_idx = 0;
    const int lane = threadIdx.x & 31;
    while (pending) {
        const int src = __ffs(pending) - 1;
        pending &= pending - 1;
        const unsigned long long bp =
            __shfl_sync(0xffffffffu, (unsigned long long)reinterpret_cast<uintptr_t>(q.bin), src);
        const int qn = __shfl_sync(0xffffffffu, q.n, src);
        const float qlx = __shfl_sync(0xffffffffu, q.lx, src);
        const int qmode = __shfl_sync(0xffffffffu, q.mode, src);
        const int idx = bound_warp(reinterpret_cast<const float*>(bp), qn, qlx, qmode != 3);
        if (lane == src) my_idx = idx;
    }
    if (q.mode != 0) r = cddt_finish(p, q, my_idx);
    return r;
}

// ------------------------------------------------------- GiantLUTCast
// discretize_theta, RangeLib.h:1834-1867 (alternate mod, cached constants, roundf)
__device__ __forceinline__ int glt_discretize(const GltDev& g, float theta, unsigned* err) {
    int it = 0;
    if (theta < 0.0f) {
        while (theta < 0.0f) {
            if (++it > kMaxWrap) { atomicOr(err, F_WRAP_BOUND); break; }
            theta = __double2float_rn(__dadd_rn((double)theta, kM2Pi));
        }
    } else if (theta > kM2PiDownF) {
        while (theta > kM2PiDownF) {
            if (++it > kMaxWrap) { atomicOr(err, F_WRAP_BOUND); break; }
            theta = __double2float_rn(__dsub_rn((double)theta, kM2Pi));
        }
    }
    const int rounded = __float2int_rz(roundf(__fmul_rn(theta, g.td_div_2pi)));
    return (int)((unsigned)rounded % g.td);
}

// GiantLUTCast::calc_range, RangeLib.h:1869-1881; NaN arguments give max_range
__device__ __forceinline__ float glt_cast(const CastParams& p, float x, float y, float heading) {
    if (isnan(x) || isnan(y) || isnan(heading)) return p.mr;
    if (x < 0.0f || x >= __int2float_rn(p.map.W) || y < 0.0f || y >= __int2float_rn(p.map.H)) return p.mr;
    const GltDev& g = p.glt;
    const int b = glt_discretize(g, heading, p.err);
    const size_t cell = (size_t)__float2int_rz(x) * p.map.H + __float2int_rz(y);
    return __fmul_rn(__int2float_rn(__ldg(g.lut + cell * g.td + b)), g.max_div_limits);
}

// one ray per (cell corner, angle bin), angle bins fastest: lut[(x * H + y) * td + i]; the march reads
// the per-cell step map (the same steps as the distance transform's, two instructions fewer)
__global__ void __launch_bounds__(256) k_glt_build(MapDev m, float mr, unsigned td, const float* __restrict__ cosv,
                                                   const float* __restrict__ sinv, float limits_div_max,
                                                   uint16_t* __restrict__ lut, long long total) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= total) return;
    const long long cell = idx / td;
    const int i = (int)(idx - cell * td);
    const int x = (int)(cell / m.H), y = (int)(cell - (long long)x * m.H);
    float r = rm_cast<DT_STEP, 0>(m, mr, __int2float_rn(x), __int2float_rn(y), __ldg(cosv + i), __ldg(sinv + i));
    r = r < mr ? r : mr;   // std::min(max_range, r)
    lut[idx] = (uint16_t)__float2uint_rz(__fmul_rn(r, limits_div_max));
}

// -------------------------------------------- CDDT radial pairs
// calc_range_pair, RangeLib.h:1521-1615: the ranges at heading and at
// heading + pi from one bin search.  A bin outside the slice gives
// (max_range, max_range) (the reference indexes it unchecked); the forward
// branch's occupancy test has no effect in the reference and is omitted.
__device__ void cddt_pair(const CastParams& p, float x, float y, float heading, float& r, float& ri) {
    const CddtDev& c = p.cddt;
    const float mr = p.mr;
    r = mr;
    ri = mr;
    if (isnan(x) || isnan(y) || isnan(heading)) return;
    int a;
    bool fl;
    cddt_discretize(c, -heading, a, fl, p.err);
    const float ca = __ldg(c.cosv + a), sa = __ldg(c.sinv + a);
    const float lx = __fsub_rn(__fmul_rn(x, ca), __fmul_rn(y, sa));
    const float ly = __fadd_rn(__fadd_rn(__fmul_rn(x, sa), __fmul_rn(y, ca)), __ldg(c.trans + a));
    const unsigned li = (unsigned)__float2int_rz(ly);
    if (li >= (unsigned)__ldg(c.widths + a)) return;
    const unsigned b = __ldg(c.slice_base + a) + li;
    const unsigned lo = __ldg(c.bin_start + b);
    const int n = (int)(__ldg(c.bin_start + b + 1) - lo);
    const float* bin = c.zeros + lo;
    const int high = n - 1;
    if (high == -1) return;
    const float first = __ldg(bin), last = __ldg(bin + high);
    if (fl) {
        if (first > lx) { ri = ref_minf(mr, __fsub_rn(first, lx)); return; }
        if (last < lx) { r = __fsub_rn(lx, last); return; }
        const bool occ = (x > -1.0f) && (y > -1.0f) && occ_at(p.map, __float2int_rz(x), __float2int_rz(y));
        if (occ) { r = 0.0f; ri = 0.0f; return; }
        const int idx = bound_g(bin, n, lx, true) - 1;   // last zero point <= lx
        r = __fsub_rn(lx, __ldg(bin + idx));
        if (idx + 1 != n) ri = __fsub_rn(__ldg(bin + idx + 1), lx);
    } else {
        if (last < lx) { ri = ref_minf(mr, __fsub_rn(lx, last)); return; }
        const int idx = bound_g(bin, n, lx, false);        // first zero point >= lx
        r = __fsub_rn(__ldg(bin + idx), lx);
        if (idx != 0) ri = __fsub_rn(lx, __ldg(bin + idx - 1));
    }
}

__global__ void k_cddt_pair(CastParams p, float x, float y, float heading, float* out) {
    float r, ri;
    cddt_pair(p, x, y, heading, r, ri);
    out[0] = r;
    out[1] = ri;
}

// ------------------------------------------------------------- dispatch
template <int KIND, int LAYOUT, int PF = 0>
__device__ __forceinline__ float cast_one(const CastParams& p, float x, float y, float h, long long ray) {
    if (KIND == K_CDDT) return cddt_cast<PF == 2>(p, x, y, h);   // PF 2: sector search
    if (KIND == K_GLT) return glt_cast(p, x, y, h);
    float c, s;
    if (p.trig) {
        c = p.trig[2 * ray];
        s = p.trig[2 * ray + 1];
    } else {
        rlc_trig::sincos_cr(h, &s, &c);
    }
    if (KIND == K_RM) return rm_cast<LAYOUT, PF>(p.map, p.mr, x, y, c, s);
    return bl_cast(p.map, p.mr, x, y, c, s, p.err);
}

// RangeLib.h:468-475: world -> grid, then calc_range(y, x, theta)
__device__ __forceinline__ void world_to_grid(const WorldDev& w, float xw, float yw, float thw,
                                              float& ax, float& ay, float& th) {
    float x = __fmul_rn(__fsub_rn(xw, w.ox), w.inv_s);
    float y = __fmul_rn(__fsub_rn(yw, w.oy), w.inv_s);
    float tmp = x;
    x = __fsub_rn(__fmul_rn(w.ca, x), __fmul_rn(w.sa, y));
    y = __fadd_rn(__fmul_rn(w.sa, tmp), __fmul_rn(w.ca, y));
    th = __fadd_rn(-thw, w.rc);
    ax = y;
    ay = x;
}

// std::min<float>(std::max<float>(v, 0.0), (float)K - 1.0), then (int)
__device__ __forceinline__ int sensor_bin(float v, int K, unsigned* err) {
    const float hi = __int2float_rn(K - 1);
    v = ref_minf(ref_maxf(v, 0.0f), hi);
    if (isnan(v)) { atomicOr(err, F_NAN_INDEX); return 0; }
    return __float2int_rz(v);
}

// Which write of calc_range_many_radial_optimized's loops stays at row
// position q: the single-cast loop (P < q < K) writes last; otherwise the
// later of pair iteration q's forward write and pair iteration q - K's
// inverse write (each pair iteration writes forward, then inverse).
// Returns 2a for the forward write of iteration a, 2a + 1 for the inverse.
__device__ __forceinline__ int radial_last_write(int q, int mp, int off) {
    int key = -1;
    if (q >= 0 && q <= mp) key = 2 * q;
    const int ai = q - off;
    if (ai >= 0 && ai <= mp && 2 * ai + 1 > key) key = 2 * ai + 1;
    return key;
}

// one thread per (particle i, loop index a), a < max(mp + 1, off)
__global__ void __launch_bounds__(256) k_cddt_radial(CastParams p, const float* __restrict__ ins,
                                                     const float* __restrict__ angles, float* __restrict__ outs,
                                                     int n, int nr, int mp, int off, int A) {
    const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= (long long)n * A) return;
    const int i = (int)(g / A), a = (int)(g - (long long)i * A);
    float ax, ay, th;
    world_to_grid(p.world, __ldg(ins + 3 * (size_t)i), __ldg(ins + 3 * (size_t)i + 1), __ldg(ins + 3 * (size_t)i + 2),
                  ax, ay, th);
    const float h = __fsub_rn(th, __ldg(angles + a));
    float* row = outs + (size_t)i * nr;
    if (a <= mp) {
        float r, ri;
        cddt_pair(p, ax, ay, h, r, ri);
        if (a < nr && radial_last_write(a, mp, off) == 2 * a) row[a] = __fmul_rn(r, p.world.s);
        const int q = a + off;
        if (q >= 0 && q < nr && !(q > mp && q < off) && radial_last_write(q, mp, off) == 2 * a + 1)
            row[q] = __fmul_rn(ri, p.world.s);
    } else if (a < off && a < nr) {
        row[a] = __fmul_rn(cddt_cast(p, ax, ay, h), p.world.s);
    }
}

// ---------------------------------------------------------------- kernels
template <int KIND, int LAYOUT, int PF, bool WORLD>
__global__ void __launch_bounds__(256) k_calc_range_many(CastParams p, const float* __restrict__ ins,
                                                         float* __restrict__ outs, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (KIND == K_CDDT && PF == 1) {   // warp-cooperative bin search: every lane of the warp takes part
        const bool act = i < n;
        float q0 = 0.0f, q1 = 0.0f, q2 = 0.0f;
        if (act) { q0 = __ldg(ins + 3 * (size_t)i); q1 = __ldg(ins + 3 * (size_t)i + 1); q2 = __ldg(ins + 3 * (size_t)i + 2); }
        float r;
        if (WORLD) {
            float ax, ay, th;
            world_to_grid(p.world, q0, q1, q2, ax, ay, th);
            r = __fmul_rn(cddt_cast_warp(p, act, ax, ay, th), p.world.s);
        } else {
            r = cddt_cast_warp(p, act, q0, q1, q2);
        }
        if (act) outs[i] = r;
        return;
    }
    if (i >= n) return;
    float q0 = __ldg(ins + 3 * (size_t)i), q1 = __ldg(ins + 3 * (size_t)i + 1), q2 = __ldg(ins + 3 * (size_t)i + 2);
    if (WORLD) {
        float ax, ay, th;
        world_to_grid(p.world, q0, q1, q2, ax, ay, th);
        outs[i] = __fmul_rn(cast_one<KIND, LAYOUT, PF>(p, ax, ay, th, i), p.world.s);
    } else {
        outs[i] = cast_one<KIND, LAYOUT, PF>(p, q0, q1, q2, i);
    }
}

// RangeLib.h:482-520: rays are particle-major, ray = i * na + a
template <int KIND, int LAYOUT, int PF>
__global__ void __launch_bounds__(256) k_repeat_angles(CastParams p, const float* __restrict__ ins,
                                                       const float* __restrict__ angles,
                                                       float* __restrict__ outs, int n, int na) {
    long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (KIND == K_CDDT && PF == 1) {   // warp-cooperative bin search
        const bool act = g < (long long)n * na;
        float ax = 0.0f, ay = 0.0f, h = 0.0f;
        if (act) {   // n * na < 2^31 (the ABI refuses larger calls): 32-bit division
            const unsigned gu = (unsigned)g, i = gu / (unsigned)na, a = gu - i * (unsigned)na;
            float th;
            world_to_grid(p.world, __ldg(ins + 3 * (size_t)i), __ldg(ins + 3 * (size_t)i + 1),
                          __ldg(ins + 3 * (size_t)i + 2), ax, ay, th);
            h = __fsub_rn(th, __ldg(angles + a));
        }
        const float r = cddt_cast_warp(p, act, ax, ay, h);
        if (act) outs[g] = __fmul_rn(r, p.world.s);
        return;
    }
    if (g >= (long long)n * na) return;
    const unsigned gu = (unsigned)g, i = gu / (unsigned)na, a = gu - i * (unsigned)na;   // n * na < 2^31
    float ax, ay, th;
    world_to_grid(p.world, __ldg(ins + 3 * (size_t)i), __ldg(ins + 3 * (size_t)i + 1),
                  __ldg(ins + 3 * (size_t)i + 2), ax, ay, th);
    float r = cast_one<KIND, LAYOUT, PF>(p, ax, ay, __fsub_rn(th, __ldg(angles + a)), g);
    outs[g] = __fmul_rn(r, p.world.s);
}

// ------------------------------------------------------------ sensor model
// The weight of a particle is the product of its beams' table values in beam
// order (RangeLib.h:533-555, 558-612), in double, exactly as the reference
// multiplies -- so weights are bit-identical.  A tile holds P particles
// and the products run one particle per lane: each double multiply
// instruction then serves up to 32 particles instead of one (the FP64 pipe
// spends the same time on a warp instruction with one active lane as with
// 32).  In eval_sensor_model's tiles the given ranges' 16-bit bins sit in
// shared memory (sdi, particle-major) beside the beams' observation bins
// (sri): (P * na + na) * 2 bytes per block; the fused update keeps each
// ray's table factor instead (k_fused).
struct TileSmem {
    uint16_t* sdi;   // [P * na] range bins
    uint16_t* sri;   // [na] observation bins
};

__host__ __device__ inline size_t tile_smem(int P, int na) {
    return (((size_t)P * na + (size_t)na) * sizeof(uint16_t) + 15) & ~(size_t)15;
}

__device__ __forceinline__ TileSmem tile_layout(unsigned char* base, int P, int na) {
    TileSmem t;
    t.sdi = reinterpret_cast<uint16_t*>(base);
    t.sri = t.sdi + (size_t)P * na;
    return t;
}

// In-order product of the table factors table[sri(a) * K + bin(a)], a = 0 ..
// na - 1, as a three-stage software pipeline over groups of kGroup beams: in
// each step the bins of group g + 2 and the factors of group g + 1 are
// requested while group g is multiplied, so the dependent bin -> factor ->
// multiply chain of one group no longer waits on memory.  Groups past na
// multiply by 1.0, which leaves every double (subnormals included) as is.
// group_bins(g, b) delivers the kGroup bins of group g (entries past na are
// not used).  Registers: 2 x kGroup doubles and 2 x kGroup bins.
template <int kGroup, class SriF, class GroupF>
__device__ __forceinline__ double product_chain(const SensorDev& sm, int na, SriF sri, GroupF group_bins) {
    unsigned bx[kGroup], by[kGroup];
    double f0[kGroup], f1[kGroup];
    const int ng = (na + kGroup - 1) / kGroup;
    auto load_bins = [&](unsigned* b, int g) {
        if (g < ng) group_bins(g, b);
    };
    auto load_factors = [&](double* f, const unsigned* b, int g) {
#pragma unroll
        for (int u = 0; u < kGroup; ++u) {
            const int a = g * kGroup + u;
            f[u] = a < na ? __ldg(sm.table + (size_t)sri(a) * sm.K + b[u]) : 1.0;
        }
    };
    auto multiply = [&](double w, const double* f) {
#pragma unroll
        for (int u = 0; u < kGroup; ++u) w = __dmul_rn(w, f[u]);
        return w;
    };
    double w = 1.0;
    load_bins(bx, 0);
    load_factors(f0, bx, 0);
    load_bins(bx, 1);
    for (int g = 0; g < ng; g += 2) {
        load_bins(by, g + 2);
        load_factors(f1, bx, g + 1);
        w = multiply(w, f0);
        if (g + 1 >= ng) break;
        load_bins(bx, g + 3);
        load_factors(f0, by, g + 2);
        w = multiply(w, f1);
    }
    return w;
}

// one lane per particle; a short unrolled gather keeps the fused kernels' registers low
__device__ __forceinline__ void tile_products(const SensorDev& sm, const TileSmem& ts, int na, int P, int first,
                                              int n, double* __restrict__ weights) {
    for (int li = threadIdx.x; li < P; li += blockDim.x) {
        const int i = first + li;
        if (i >= n) continue;
        const uint16_t* row = ts.sdi + (size_t)li * na;
        double w = 1.0;
#pragma unroll 8
        for (int a = 0; a < na; ++a) w = __dmul_rn(w, __ldg(sm.table + (size_t)ts.sri[a] * sm.K + row[a]));
        weights[i] = w;
    }
}

__device__ __forceinline__ void tile_obs_bins(const CastParams& p, const SensorDev& sm, const float* __restrict__ obs,
                                              int na, uint16_t* sri) {
    for (int a = threadIdx.x; a < na; a += blockDim.x)
        sri[a] = (uint16_t)sensor_bin(__fmul_rn(__ldg(obs + a), p.world.inv_s), sm.K, p.err);
}

// RangeLib.h:533-555 on given ranges (world units)
__global__ void __launch_bounds__(512) k_eval_sensor(CastParams p, SensorDev sm, const float* __restrict__ obs,
                                                     const float* __restrict__ ranges, double* __restrict__ outs,
                                                     int na, int n, int P) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const TileSmem ts = tile_layout(smem_raw, P, na);
    const int first = blockIdx.x * P;
    tile_obs_bins(p, sm, obs, na, ts.sri);
    const int nr = P * na;
    for (int r = threadIdx.x; r < nr; r += blockDim.x) {
        int li = r / na, a = r - li * na, i = first + li;
        if (i < n) ts.sdi[r] = (uint16_t)sensor_bin(__fmul_rn(__ldg(ranges + (size_t)i * na + a), p.world.inv_s), sm.K, p.err);
    }
    __syncthreads();
    tile_products(sm, ts, na, P, first, n, outs);
}

// range of ray (particle i, beam a) in pixels (RangeLib.h:558-612)
template <int KIND, int LAYOUT, int PF>
__device__ __forceinline__ float cast_ray(const CastParams& p, const float* __restrict__ ins,
                                          const float* __restrict__ angles, int i, int a, int na, int layout, int pf) {
    float ax, ay, th;
    world_to_grid(p.world, __ldg(ins + 3 * (size_t)i), __ldg(ins + 3 * (size_t)i + 1), __ldg(ins + 3 * (size_t)i + 2),
                  ax, ay, th);
    const long long ray = (long long)i * na + a;
    const float h = __fsub_rn(th, __ldg(angles + a));
    if (KIND >= 0) return cast_one<KIND, LAYOUT, PF>(p, ax, ay, h, ray);
    if (KIND == kRmOnly) return cast_one<K_RM, LAYOUT, PF>(p, ax, ay, h, ray);   // every filter ray-marches
    // mixed kinds: dispatch at run time
    if (p.kind == K_RM) {
        if (layout == DT_RUNS)
            return pf ? cast_one<K_RM, DT_RUNS, kPrefetch>(p, ax, ay, h, ray) : cast_one<K_RM, DT_RUNS, 0>(p, ax, ay, h, ray);
        if (layout == DT_STEP)
            return pf ? cast_one<K_RM, DT_STEP, kPrefetch>(p, ax, ay, h, ray) : cast_one<K_RM, DT_STEP, 0>(p, ax, ay, h, ray);
        if (layout == DT_U16)
            return pf ? cast_one<K_RM, DT_U16, kPrefetch>(p, ax, ay, h, ray) : cast_one<K_RM, DT_U16, 0>(p, ax, ay, h, ray);
        if (layout == DT_TILED)
            return pf ? cast_one<K_RM, DT_TILED, kPrefetch>(p, ax, ay, h, ray)
                      : cast_one<K_RM, DT_TILED, 0>(p, ax, ay, h, ray);
        return pf ? cast_one<K_RM, DT_LINEAR, kPrefetch>(p, ax, ay, h, ray) : cast_one<K_RM, DT_LINEAR, 0>(p, ax, ay, h, ray);
    }
    if (p.kind == K_BL) return cast_one<K_BL, DT_LINEAR, 0>(p, ax, ay, h, ray);
    if (p.kind == K_GLT) return cast_one<K_GLT, DT_LINEAR, 0>(p, ax, ay, h, ray);
    return cast_one<K_CDDT, DT_LINEAR, 0>(p, ax, ay, h, ray);
}

// Fused update, one tile of P particles per block.  Each ray's thread casts the ray, bins it
// and reads its table factor -- row: the beam's observation bin, column: the range bin -- into
// shared memory (sf, particle-major, double); after the block's barrier the P particles' lanes
// multiply their factors in beam order.  The factor reads run beside the other rays' marches,
// one per ray, instead of as a chain of dependent groups after the barrier: in this one-wave
// launch on a flushed L2 that chain sat on the step's critical path.  Shared memory per block:
// P * na * 8 bytes.  The march kernels are held to 32 registers (the bounds' 4 blocks of 512
// threads), so that a particle-filter step's blocks of 128 threads stay resident at 16 per SM
// in one wave; the CDDT searches keep their registers.
template <int KIND, int LAYOUT, int PF>
__global__ void __launch_bounds__(512, KIND == K_CDDT ? 1 : 4) k_fused(CastParams p, SensorDev sm, const float* __restrict__ ins,
                                               const float* __restrict__ angles, const float* __restrict__ obs,
                                               double* __restrict__ weights, int n, int na, int P) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double* sf = reinterpret_cast<double*>(smem_raw);
    const int first = blockIdx.x * P, nr = P * na;
    const float inv_na = __frcp_rn(__int2float_rn(na));
    for (int r = threadIdx.x; r < nr; r += blockDim.x) {
        const int li = div_small(r, na, inv_na), a = r - li * na, i = first + li;
        if (i < n) {
            const int ob = sensor_bin(__fmul_rn(__ldg(obs + a), p.world.inv_s), sm.K, p.err);
            const float d = cast_ray<KIND, LAYOUT, PF>(p, ins, angles, i, a, na, LAYOUT, PF);
            sf[r] = __ldg(sm.table + (size_t)ob * sm.K + sensor_bin(d, sm.K, p.err));
        }
    }
    __syncthreads();
    for (int li = threadIdx.x; li < P; li += blockDim.x) {
        const int i = first + li;
        if (i >= n) continue;
        const double* f = sf + (size_t)li * na;
        double w = 1.0;
#pragma unroll 8
        for (int a = 0; a < na; ++a) w = __dmul_rn(w, f[a]);
        weights[i] = w;
    }
}

// ------------------------------------------------- persistent multi-filter
// Every block loops: take the next tile index from the device queue and
// cast the tile's rays (P particles of one filter) into the filter's range
// bins in global memory; warps take the rays 32 at a time from a
// shared-memory counter.  The products of a tile's particles (in beam order,
// up to 32 particles per lane set) are run by warp 0 while the other warps
// cast the block's next tile -- a product chain is as long as the tile's
// beam count in dependent double multiplies, and would otherwise idle the
// block -- and warp 0 joins the cast when it is done.  Filters are stored in
// descending per-tile cost, so heavy tiles are handed out first.  There is
// no waiting on other blocks: a block that finds the queue exhausted
// multiplies its last tile and exits.
// the four range bins of beams 4g .. 4g + 3 of tile particle li: one 8-byte read (batch bin layout)
__device__ __forceinline__ void tile_bins4(const uint16_t* tile, int P, int li, int g, unsigned* b) {
    const uint2 v = *reinterpret_cast<const uint2*>(tile + ((size_t)g * P + li) * 4);
    b[0] = v.x & 0xFFFFu;
    b[1] = v.x >> 16;
    b[2] = v.y & 0xFFFFu;
    b[3] = v.y >> 16;
}

__device__ __forceinline__ void batch_products(const FilterDev& F, int tile, int np) {
    const int lane = threadIdx.x & 31;
    const uint16_t* obs_bins = F.obs_bins;
    const uint16_t* tb = F.bins + batch_tile_offset(F, tile);
    const int P = F.ppb, first = tile * P;
    for (int li = lane; li < np; li += 32) {
        F.weights[first + li] = product_chain<4>(
            F.sm, F.na, [&](int a) { return (unsigned)__ldg(obs_bins + a); },
            [&](int g, unsigned* b) { tile_bins4(tb, P, li, g, b); });
    }
}

// ray r of a tile: its range into the filter's ranges (if kept) and its bin into the tile's bins
__device__ __forceinline__ void batch_store(const FilterDev& F, int first, uint16_t* bins, int r, float d) {
    const int P = F.ppb, na = F.na;
    const int li = div_small(r, na, F.inv_na), a = r - li * na;
    if (F.ranges) F.ranges[(size_t)(first + li) * na + a] = d;
    bins[((size_t)(a >> 2) * P + li) * 4 + (a & 3)] = (uint16_t)sensor_bin(d, F.sm.K, F.p.err);
}

// Ray (particle i, beam a) of a ray-marching filter at the start of its march (RangeLib.h:558-612,
// 927-931); r is the tile's index of the ray.  The particle's grid-frame pose comes from its
// record; the ray's cos/sin from the caller's override, else from the float pairs of the particle
// heading's and the beam angle's sin and cos (rlc_trig::sincos_diff: the correctly rounded values
// of the ray's heading fl(th - a), for about a third of the instructions of computing them from
// the heading), else -- where no pairs exist or their rounding is not certain -- from the heading.
__device__ __forceinline__ RmRay rm_ray_start(const FilterDev& F, int i, int a, int r) {
    const float4 pose = __ldg(F.part_rec + 2 * (size_t)i);
    const float ang = __ldg(F.angles + a);
    const float h = __fsub_rn(pose.z, ang);
    float c, s;
    if (F.p.trig) {
        const long long ray = (long long)i * F.na + a;
        c = F.p.trig[2 * ray];
        s = F.p.trig[2 * ray + 1];
    } else {
        const float4 pt = __ldg(F.part_rec + 2 * (size_t)i + 1), bt = __ldg(F.beam_rec + a);
        if (isnan(pt.x) || isnan(bt.x) ||
            !rlc_trig::sincos_diff(pose.z, ang, rlc_trig::F2{pt.x, pt.y}, rlc_trig::F2{pt.z, pt.w},
                                   rlc_trig::F2{bt.x, bt.y}, rlc_trig::F2{bt.z, bt.w}, &s, &c))
            rlc_trig::sincos_cr(h, &s, &c);
    }
    return RmRay{pose.x, pose.y, c, s, 0.0f, -1.0f, 0, r};
}

// A tile's rays in a ray-marching batch, with a march budget.  A warp takes 32 rays at a time;
// each lane marches its ray for at most kBatchBudget rounds, and rays that have not ended are
// handed on: their march state goes to the warp's slots in shared memory, and whenever 32 are
// waiting the warp marches them to their ends together.  A warp's time per 32 rays is its
// slowest lane's; the handed-on rays -- the long ones -- now share warps with one another instead
// of holding up 31 short ones (a CPU count over the uneven batch: 15 % fewer warp rounds at a
// budget of 16; measured on the 32-filter batch: 3.09 -> 2.84 ms, against 2.87 / 2.92 / 2.99 ms
// at budgets 12 / 10 / 8 and 2.85 / 3.22 ms at 20 / 24).  The saved state is the march's own
// (RmRay), so every range is the one the uninterrupted march gives.
constexpr int kBatchBudget = 16;   // march rounds before a ray is handed on
constexpr int kBatchSlots = 64;    // handed-on rays a warp can hold (at most 31 + 32 wait at once)

template <int LAYOUT, int PF>
__device__ __forceinline__ void batch_cast_budgeted(const FilterDev& F, int first, int nr, uint16_t* bins,
                                                    RmRay* slots, unsigned* next) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const unsigned below = (1u << lane) - 1u;
    const CastParams& p = F.p;
    int held = 0;        // handed-on rays in the warp's slots (the same in every lane)
    bool fresh = true;   // the tile still hands out rays
    for (;;) {
        unsigned base = 0u;
        if (fresh) {
            if (lane == 0) base = atomicAdd(next, 32u);
            base = __shfl_sync(full, base, 0);
            fresh = base < (unsigned)nr;
        }
        if (!fresh) {   // the tile's rays are handed out: finish the warp's handed-on rays
            if (held == 0) return;
            const int take = min(held, 32);
            __syncwarp();
            if (lane < take) {
                RmRay q = slots[held - take + lane];
                float d = p.mr;
                rm_advance<LAYOUT, PF, false>(p.map, p.mr, q, 0, &d, nullptr);
                batch_store(F, first, bins, q.r, d);
            }
            held -= take;
            continue;
        }
        const int r = (int)base + lane;
        bool pending = false;
        RmRay q;
        if (r < nr) {
            const int li = div_small(r, F.na, F.inv_na), a = r - li * F.na;
            q = rm_ray_start(F, first + li, a, r);
            float d = p.mr;
            bool done = true;   // NaN arguments and max_range <= 0 give max_range (rm_cast)
            if (!(isnan(q.x0) || isnan(q.y0) || isnan(q.c) || isnan(q.s)) && 0.0f < p.mr)
                done = rm_advance<LAYOUT, PF, true>(p.map, p.mr, q, kBatchBudget, &d, nullptr);
            if (done) batch_store(F, first, bins, r, d); else pending = true;
        }
        const unsigned pm = __ballot_sync(full, pending);
        if (pending) slots[held + __popc(pm & below)] = q;
        held += __popc(pm);
        if (held >= 32) {   // 32 handed-on rays: march them to their ends together
            __syncwarp();
            RmRay h = slots[held - 32 + lane];
            held -= 32;
            __syncwarp();   // every lane has read its slot before the next rays land there
            float d = p.mr;
            rm_advance<LAYOUT, PF, false>(p.map, p.mr, h, 0, &d, nullptr);
            batch_store(F, first, bins, h.r, d);
        }
    }
}

template <int MODE, int LAYOUT, int PF, bool SEPARATE>
__global__ void __launch_bounds__(512, 4) k_batch(const FilterDev* __restrict__ filters, int nf, unsigned total_tiles,
                                               unsigned* __restrict__ queue) {
    __shared__ unsigned s_tile, s_next;
    __shared__ int s_f;
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const bool mult = threadIdx.x < 32;   // warp 0 multiplies the previous tile
    int prev_f = -1, prev_tile = 0, prev_np = 0;
    for (;;) {
        if (threadIdx.x == 0) {
            const unsigned t = atomicAdd(queue, 1u);
            s_tile = t;
            int lo = 0, hi = nf - 1;   // last filter with tile_begin <= t
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (filters[mid].tile_begin <= t) lo = mid; else hi = mid - 1;
            }
            s_f = lo;
            s_next = 0u;
        }
        __syncthreads();
        const unsigned t = s_tile;
        const int f = s_f;
        if (!SEPARATE && mult && prev_f >= 0) batch_products(filters[prev_f], prev_tile, prev_np);
        if (t >= total_tiles) break;
        const FilterDev& F = filters[f];
        const int P = F.ppb, na = F.na, n = F.n;
        const int tile = (int)(t - F.tile_begin), first = tile * P;
        const int nr = min(P, n - first) * na;
        uint16_t* bins = F.bins + batch_tile_offset(F, tile);
        if (MODE == kRmOnly) {
            extern __shared__ __align__(16) unsigned char smem_raw[];
            batch_cast_budgeted<LAYOUT, PF>(F, first, nr, bins,
                                            reinterpret_cast<RmRay*>(smem_raw) + (threadIdx.x >> 5) * kBatchSlots,
                                            &s_next);
        } else {
            for (;;) {
                unsigned base = 0u;
                if (lane == 0) base = atomicAdd(&s_next, 32u);
                base = __shfl_sync(full, base, 0);
                if (base >= (unsigned)nr) break;
                const int r = (int)base + lane;
                if (r < nr) {
                    const int li = div_small(r, na, F.inv_na), a = r - li * na;
                    const float d =
                        cast_ray<MODE, LAYOUT, PF>(F.p, F.ins, F.angles, first + li, a, na, F.layout, F.prefetch);
                    batch_store(F, first, bins, r, d);
                }
            }
        }
        __syncthreads();   // the tile's bins are written; s_tile, s_f and s_next may be reused
        prev_f = f;
        prev_tile = tile;
        prev_np = min(P, n - first);
    }
}


// Products of every particle of the batch in one launch after the cast (the
// alternative to k_batch's overlapped products): one thread per particle,
// 32 particles per warp, the bins read back from global memory.
__global__ void __launch_bounds__(256) k_batch_products(const FilterDev* __restrict__ filters, int nf,
                                                        unsigned total_particles) {
    const unsigned g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= total_particles) return;
    int lo = 0, hi = nf - 1;   // last filter with part_begin <= g
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (filters[mid].part_begin <= g) lo = mid; else hi = mid - 1;
    }
    const FilterDev& F = filters[lo];
    const int i = (int)(g - F.part_begin);
    const int P = F.ppb, tile = i / P, li = i - tile * P;
    const uint16_t* obs_bins = F.obs_bins;
    const uint16_t* tb = F.bins + batch_tile_offset(F, tile);
    // groups of 8 beams (two 8-byte bin reads; a last half group past the tile's bins reads none):
    // twice the factor reads in flight of the overlapped products' groups of 4, 1.4 % of the step
    const int bin_groups = (F.na + 3) >> 2;
    F.weights[i] = product_chain<8>(
        F.sm, F.na, [&](int a) { return (unsigned)__ldg(obs_bins + a); },
        [&](int gr, unsigned* b) {
            tile_bins4(tb, P, li, 2 * gr, b);
            if (2 * gr + 1 < bin_groups) tile_bins4(tb, P, li, 2 * gr + 1, b + 4);
            else b[4] = b[5] = b[6] = b[7] = 0u;
        });
}

// the observation bin of every beam of every filter, once per batch run (products read them)
// (ray-marching batches: and every beam's record -- the angle's sin and cos as float pairs)
__global__ void k_batch_obs_bins(const FilterDev* __restrict__ filters, bool records) {
    const FilterDev& F = filters[blockIdx.x];
    for (int a = threadIdx.x; a < F.na; a += blockDim.x) {
        F.obs_bins[a] = (uint16_t)sensor_bin(__fmul_rn(__ldg(F.obs + a), F.p.world.inv_s), F.sm.K, F.p.err);
        if (records) {
            rlc_trig::F2 sn, cs;
            F.beam_rec[a] = rlc_trig::sincos_pairs(__ldg(F.angles + a), &sn, &cs) ? make_float4(sn.h, sn.l, cs.h, cs.l)
                                                                                    : make_float4(__int_as_float(0x7fc00000), 0.0f, 0.0f, 0.0f);
        }
    }
}

// Every particle's record of a ray-marching batch, once per run: the world -> grid transform of
// its pose (RangeLib.h:468-475) and, unless the filter has a trig override, its heading's sin and
// cos as float pairs; one thread per particle of the batch.
__global__ void __launch_bounds__(256) k_batch_particles(const FilterDev* __restrict__ filters, int nf,
                                                         unsigned total_particles) {
    const unsigned g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= total_particles) return;
    int lo = 0, hi = nf - 1;   // last filter with part_begin <= g
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (filters[mid].part_begin <= g) lo = mid; else hi = mid - 1;
    }
    const FilterDev& F = filters[lo];
    const size_t i = g - F.part_begin;
    float ax, ay, th;
    world_to_grid(F.p.world, __ldg(F.ins + 3 * i), __ldg(F.ins + 3 * i + 1), __ldg(F.ins + 3 * i + 2), ax, ay, th);
    F.part_rec[2 * i] = make_float4(ax, ay, th, 0.0f);
    rlc_trig::F2 sn, cs;
    F.part_rec[2 * i + 1] = !F.p.trig && rlc_trig::sincos_pairs(th, &sn, &cs)
                                ? make_float4(sn.h, sn.l, cs.h, cs.l)
                                : make_float4(__int_as_float(0x7fc00000), 0.0f, 0.0f, 0.0f);
}


// ------------------------------------------- beam-major fused update (staged)
// One block per (beam a, chunk of particles): its rays start near the same
// particle cluster and share a heading, so they sweep one bundle.  The block
// copies the 8x8 tiles of the 8-bit squared distance transform that cover
// the bundle's bounding box (capped at kStagedWindow bytes, shrunk around
// its centre beyond that) into shared memory, with a 256-entry table of the
// step max(sqrtf(v) * 0.999f, 1) of each d^2 = v.  Cells inside the window
// with v <= 254 -- those next to walls, where long rays take their many
// short steps -- are then read from shared memory; v = 255 cells and cells
// outside the window read the float distance transform.  sqrtf(v) is the
// distance transform's value exactly, so every step equals the reference's.
constexpr int kStagedThreads = 1024;
constexpr int kStagedWindow = 216 * 1024;

__global__ void __launch_bounds__(kStagedThreads, 1) k_bm_cast(CastParams p, SensorDev sm, const float* __restrict__ ins,
                                                              const float* __restrict__ angles, int n, int na, int P,
                                                              uint16_t* __restrict__ bins, int cap_tiles) {
    extern __shared__ __align__(16) uint8_t smem[];
    float* step_tab = reinterpret_cast<float*>(smem);   // [256]
    uint8_t* win = smem + 1024;
    __shared__ int bb[4];
    const MapDev& m = p.map;
    const int a = blockIdx.x;
    const int first = blockIdx.y * P, last = min(n, first + P);
    const float ang = __ldg(angles + a);
    for (int v = threadIdx.x; v < 256; v += blockDim.x)
        step_tab[v] = ref_maxf(__fmul_rn(__fsqrt_rn(__uint2float_rn(v)), 0.999f), 1.0f);
    if (threadIdx.x == 0) { bb[0] = INT_MAX; bb[1] = INT_MIN; bb[2] = INT_MAX; bb[3] = INT_MIN; }
    __syncthreads();
    // bounding box of the bundle's segments [start, start + max_range * dir]
    int xmn = INT_MAX, xmx = INT_MIN, ymn = INT_MAX, ymx = INT_MIN;
    for (int i = first + threadIdx.x; i < last; i += blockDim.x) {
        float ax, ay, th;
        world_to_grid(p.world, __ldg(ins + 3 * (size_t)i), __ldg(ins + 3 * (size_t)i + 1),
                      __ldg(ins + 3 * (size_t)i + 2), ax, ay, th);
        float c, s;
        rlc_trig::sincos_cr(__fsub_rn(th, ang), &s, &c);
        const float ex = ax + p.mr * c, ey = ay + p.mr * s;
        if (!(isfinite(ax) && isfinite(ay) && isfinite(ex) && isfinite(ey))) continue;
        const float lx = fminf(fmaxf(fminf(ax, ex), -1e6f), 1e6f), hx = fminf(fmaxf(fmaxf(ax, ex), -1e6f), 1e6f);
        const float ly = fminf(fmaxf(fminf(ay, ey), -1e6f), 1e6f), hy = fminf(fmaxf(fmaxf(ay, ey), -1e6f), 1e6f);
        xmn = min(xmn, (int)floorf(lx) - 1);
        xmx = max(xmx, (int)ceilf(hx) + 1);
        ymn = min(ymn, (int)floorf(ly) - 1);
        ymx = max(ymx, (int)ceilf(hy) + 1);
    }
    for (int o = 16; o; o >>= 1) {
        xmn = min(xmn, __shfl_xor_sync(0xffffffffu, xmn, o));
        xmx = max(xmx, __shfl_xor_sync(0xffffffffu, xmx, o));
        ymn = min(ymn, __shfl_xor_sync(0xffffffffu, ymn, o));
        ymx = max(ymx, __shfl_xor_sync(0xffffffffu, ymx, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMin(&bb[0], xmn);
        atomicMax(&bb[1], xmx);
        atomicMin(&bb[2], ymn);
        atomicMax(&bb[3], ymx);
    }
    __syncthreads();
    const int TX = (m.W + 7) >> 3, TY = m.tiles_y;
    int tx0 = max(0, bb[0] >> 3), tx1 = min(TX - 1, bb[1] >> 3);
    int ty0 = max(0, bb[2] >> 3), ty1 = min(TY - 1, bb[3] >> 3);
    int ntx = tx1 - tx0 + 1, nty = ty1 - ty0 + 1;
    if (ntx <= 0 || nty <= 0) { ntx = 0; nty = 0; }
    if (ntx * nty > cap_tiles) {   // shrink around the box centre
        const float sc = sqrtf((float)cap_tiles / (float)(ntx * nty));
        int nx = max(1, min(ntx, (int)(ntx * sc)));
        int ny = max(1, min(nty, cap_tiles / nx));
        tx0 += (ntx - nx) / 2;
        ty0 += (nty - ny) / 2;
        ntx = nx;
        nty = ny;
    }
    // copy the window's tiles: rows of nty consecutive tiles are contiguous in global memory
    const int nvec = ntx * nty * 4;
    for (int v = threadIdx.x; v < nvec; v += blockDim.x) {
        const int t = v >> 2, part = v & 3;
        const int ltx = t / nty, lty = t - ltx * nty;
        const uint4 val = __ldg(reinterpret_cast<const uint4*>(m.dt8 + ((size_t)(tx0 + ltx) * TY + ty0 + lty) * 64) + part);
        reinterpret_cast<uint4*>(win)[v] = val;
    }
    __syncthreads();
    // march every ray of the block
    for (int i = first + threadIdx.x; i < last; i += blockDim.x) {
        float x0, y0, th;
        world_to_grid(p.world, __ldg(ins + 3 * (size_t)i), __ldg(ins + 3 * (size_t)i + 1),
                      __ldg(ins + 3 * (size_t)i + 2), x0, y0, th);
        const long long ray = (long long)i * na + a;
        float c, s;
        if (p.trig) { c = p.trig[2 * ray]; s = p.trig[2 * ray + 1]; } else rlc_trig::sincos_cr(__fsub_rn(th, ang), &s, &c);
        float out = p.mr;
        if (!(isnan(x0) || isnan(y0) || isnan(c) || isnan(s))) {
            float t = 0.0f;
            while (t < p.mr) {
                const int px = __float2int_rz(__fadd_rn(x0, __fmul_rn(c, t)));
                const int py = __float2int_rz(__fadd_rn(y0, __fmul_rn(s, t)));
                if ((unsigned)px >= (unsigned)m.W || (unsigned)py >= (unsigned)m.H) break;
                const int ltx = (px >> 3) - tx0, lty = (py >> 3) - ty0;
                unsigned v = 255u;
                if ((unsigned)ltx < (unsigned)ntx && (unsigned)lty < (unsigned)nty)
                    v = win[((ltx * nty + lty) << 6) | ((px & 7) << 3) | (py & 7)];
                bool hit;
                float step;
                if (v != 255u) {
                    hit = v == 0u;
                    step = step_tab[v];
                } else {
                    const float d = __ldg(m.dt + (size_t)px * m.H + py);
                    hit = d <= 0.0f;
                    step = ref_maxf(__fmul_rn(d, 0.999f), 1.0f);
                }
                if (hit) {
                    const float xd = __fsub_rn(__int2float_rn(px), x0), yd = __fsub_rn(__int2float_rn(py), y0);
                    out = __fsqrt_rn(__fadd_rn(__fmul_rn(xd, xd), __fmul_rn(yd, yd)));
                    break;
                }
                t = __fadd_rn(t, step);
            }
        }
        bins[(size_t)a * n + i] = (uint16_t)sensor_bin(out, sm.K, p.err);
    }
}

// per-particle products of the beam-major bins, in beam order: the block
// gathers the table factors of its PB particles into shared memory (beam-
// major, all gathers in flight at once), then one lane per particle multiplies
__global__ void __launch_bounds__(128) k_bm_weights(CastParams p, SensorDev sm, const float* __restrict__ obs,
                                                    const uint16_t* __restrict__ bins, int n, int na, int PB,
                                                    double* __restrict__ weights) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double* sdv = reinterpret_cast<double*>(smem_raw);
    uint16_t* sri = reinterpret_cast<uint16_t*>(smem_raw + (size_t)PB * na * sizeof(double));
    for (int a = threadIdx.x; a < na; a += blockDim.x)
        sri[a] = (uint16_t)sensor_bin(__fmul_rn(__ldg(obs + a), p.world.inv_s), sm.K, p.err);
    __syncthreads();
    const int first = blockIdx.x * PB;
    const int np = min(PB, n - first);
    const int nr = np * na;
    constexpr int kBatch = 4;
    for (int r0 = threadIdx.x; r0 < nr; r0 += kBatch * blockDim.x) {
        double v[kBatch];
#pragma unroll
        for (int u = 0; u < kBatch; ++u) {
            const int r = r0 + u * blockDim.x;
            if (r < nr) {
                const int a = r / np, li = r - a * np;
                v[u] = __ldg(sm.table + (size_t)sri[a] * sm.K + __ldg(bins + (size_t)a * n + first + li));
            }
        }
#pragma unroll
        for (int u = 0; u < kBatch; ++u) {
            const int r = r0 + u * blockDim.x;
            if (r < nr) {
                const int a = r / np, li = r - a * np;
                sdv[(size_t)a * PB + li] = v[u];
            }
        }
    }
    __syncthreads();
    if (threadIdx.x < np) {
        double w = 1.0;
#pragma unroll 8
        for (int a = 0; a < na; ++a) w = __dmul_rn(w, sdv[(size_t)a * PB + threadIdx.x]);
        weights[first + threadIdx.x] = w;
    }
}

// Diagnostic: march steps (RM: distance-transform reads; BL: cells tested)
// of the world-frame repeat-angle rays, summed into *total.  Same arithmetic
// as the casting kernels; used to state the algorithmic bytes of a workload.
template <int KIND>
__global__ void __launch_bounds__(256) k_count_steps(CastParams p, const float* __restrict__ ins,
                                                     const float* __restrict__ angles, int n, int na,
                                                     unsigned long long* total) {
    long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    int steps = 0;
    if (g < (long long)n * na) {
        int i = (int)(g / na), a = (int)(g - (long long)i * na);
        float ax, ay, th;
        world_to_grid(p.world, ins[3 * (size_t)i], ins[3 * (size_t)i + 1], ins[3 * (size_t)i + 2], ax, ay, th);
        float h = __fsub_rn(th, angles[a]);
        float c, s;
        if (p.trig) { c = p.trig[2 * g]; s = p.trig[2 * g + 1]; } else rlc_trig::sincos_cr(h, &s, &c);
        if (KIND == K_RM) rm_cast<DT_LINEAR>(p.map, p.mr, ax, ay, c, s, &steps);
        else bl_cast(p.map, p.mr, ax, ay, c, s, p.err, &steps);
    }
    for (int o = 16; o; o >>= 1) steps += __shfl_xor_sync(0xffffffffu, steps, o);
    if ((threadIdx.x & 31) == 0 && steps) atomicAdd(total, (unsigned long long)steps);
}

inline unsigned blocks_for(long long n, int b) { return (unsigned)((n + b - 1) / b); }

template <template <int, int, int> class F, class... Args>
cudaError_t dispatch(int kind, int layout, int pf, Args... args) {
    if (kind == K_RM) {
        if (pf) {
            if (layout == DT_RUNS) return F<K_RM, DT_RUNS, kPrefetch>::run(args...);
            if (layout == DT_STEP) return F<K_RM, DT_STEP, kPrefetch>::run(args...);
            if (layout == DT_U16) return F<K_RM, DT_U16, kPrefetch>::run(args...);
            if (layout == DT_TILED) return F<K_RM, DT_TILED, kPrefetch>::run(args...);
            return F<K_RM, DT_LINEAR, kPrefetch>::run(args...);
        }
        if (layout == DT_RUNS) return F<K_RM, DT_RUNS, 0>::run(args...);
        if (layout == DT_STEP) return F<K_RM, DT_STEP, 0>::run(args...);
        if (layout == DT_U16) return F<K_RM, DT_U16, 0>::run(args...);
        if (layout == DT_TILED) return F<K_RM, DT_TILED, 0>::run(args...);
        return F<K_RM, DT_LINEAR, 0>::run(args...);
    }
    if (kind == K_BL) return F<K_BL, DT_LINEAR, 0>::run(args...);
    if (kind == K_GLT) return F<K_GLT, DT_LINEAR, 0>::run(args...);
    if (pf == 1) return F<K_CDDT, DT_LINEAR, 1>::run(args...);   // warp-cooperative bin search
    if (pf == 2) return F<K_CDDT, DT_LINEAR, 2>::run(args...);   // sector search
    return F<K_CDDT, DT_LINEAR, 0>::run(args...);
}

template <int KIND, int LAYOUT, int PF>
struct RunMany {
    static cudaError_t run(const CastParams& p, bool world, const float* ins, float* outs, int n, cudaStream_t s) {
        if (n <= 0) return cudaSuccess;
        if (world) k_calc_range_many<KIND, LAYOUT, PF, true><<<blocks_for(n, 256), 256, 0, s>>>(p, ins, outs, n);
        else k_calc_range_many<KIND, LAYOUT, PF, false><<<blocks_for(n, 256), 256, 0, s>>>(p, ins, outs, n);
        return cudaGetLastError();
    }
};

template <int KIND, int LAYOUT, int PF>
struct RunAngles {
    static cudaError_t run(const CastParams& p, const float* ins, const float* angles, float* outs, int n, int na,
                           cudaStream_t s) {
        long long total = (long long)n * na;
        if (total <= 0) return cudaSuccess;
        k_repeat_angles<KIND, LAYOUT, PF><<<blocks_for(total, 256), 256, 0, s>>>(p, ins, angles, outs, n, na);
        return cudaGetLastError();
    }
};

// particles per tile (P) and threads per block: P = tile if given, else the
// most particles whose rays fit one ray per thread; P is capped so that the
// tile's per-ray entries (ray_bytes each: a 16-bit bin, or the fused update's
// 8-byte factor) and the beams' 16-bit observation bins fit kTileSmem bytes
constexpr size_t kTileSmem = 48 * 1024;
inline void product_shape(int na, int block, int tile, int& P, int& threads, size_t ray_bytes = sizeof(uint16_t)) {
    if (block <= 0) block = 256;
    if (na <= 0) { P = block; threads = block; return; }   // empty product: weight 1.0
    P = tile > 0 ? tile : (na >= block ? 1 : block / na);
    int cap = (int)((kTileSmem - (size_t)na * sizeof(uint16_t)) / ((size_t)na * ray_bytes));
    if (cap < 1) cap = 1;
    if (P > cap) P = cap;
    int nr = P * na;
    threads = nr >= block ? block : ((nr + 31) / 32) * 32;
    if (threads < 32) threads = 32;
}

template <class K>
cudaError_t set_smem(K kernel, size_t bytes) {
    if (bytes <= 48 * 1024) return cudaSuccess;
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

template <int KIND, int LAYOUT, int PF>
struct RunFused {
    static cudaError_t run(const CastParams& p, const SensorDev& sm, const float* ins, const float* angles,
                           const float* obs, double* w, int n, int na, int block, int tile, cudaStream_t s) {
        if (n <= 0) return cudaSuccess;
        int P, threads;
        product_shape(na, block, tile, P, threads, sizeof(double));
        const size_t smem = (size_t)P * na * sizeof(double);
        cudaError_t e = set_smem(k_fused<KIND, LAYOUT, PF>, smem);
        if (e != cudaSuccess) return e;
        k_fused<KIND, LAYOUT, PF><<<blocks_for(n, P), threads, smem, s>>>(p, sm, ins, angles, obs, w, n, na, P);
        return cudaGetLastError();
    }
};

}  // namespace

cudaError_t launch_calc_range_many(const CastParams& p, int layout, int pf, bool world, const float* ins,
                                   float* outs, int n, cudaStream_t s) {
    return dispatch<RunMany>(p.kind, layout, pf, p, world, ins, outs, n, s);
}

cudaError_t launch_repeat_angles(const CastParams& p, int layout, int pf, const float* ins, const float* angles,
                                 float* outs, int n, int na, cudaStream_t s) {
    return dispatch<RunAngles>(p.kind, layout, pf, p, ins, angles, outs, n, na, s);
}

cudaError_t launch_eval_sensor(const CastParams& p, const SensorDev& sm, const float* obs, const float* ranges,
                               double* outs, int na, int n, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    int P, threads;
    product_shape(na, 256, 0, P, threads);
    size_t smem = tile_smem(P, na);
    cudaError_t e = set_smem(k_eval_sensor, smem);
    if (e != cudaSuccess) return e;
    k_eval_sensor<<<blocks_for(n, P), threads, smem, s>>>(p, sm, obs, ranges, outs, na, n, P);
    return cudaGetLastError();
}

cudaError_t launch_fused(const CastParams& p, int layout, int pf, const SensorDev& sm, const float* ins,
                         const float* angles, const float* obs, double* weights, int n, int na, int block, int tile,
                         cudaStream_t s) {
    return dispatch<RunFused>(p.kind, layout, pf, p, sm, ins, angles, obs, weights, n, na, block, tile, s);
}

int tile_particles(int na, int block, int tile) {
    int P, threads;
    product_shape(na, block, tile, P, threads, sizeof(double));
    return P;
}


cudaError_t launch_count_steps(const CastParams& p, const float* ins, const float* angles, int n, int na,
                               unsigned long long* total, cudaStream_t s) {
    long long rays = (long long)n * na;
    if (rays <= 0) return cudaSuccess;
    if (p.kind == K_RM) k_count_steps<K_RM><<<blocks_for(rays, 256), 256, 0, s>>>(p, ins, angles, n, na, total);
    else if (p.kind == K_BL) k_count_steps<K_BL><<<blocks_for(rays, 256), 256, 0, s>>>(p, ins, angles, n, na, total);
    else return cudaErrorInvalidValue;
    return cudaGetLastError();
}

// the per-ray cos/sin of the casts (rlc_trig::sincos_cr) for given arguments
__global__ void __launch_bounds__(256) k_trig_eval(const float* __restrict__ x, float2* __restrict__ sc, long long n) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        float s, c;
        rlc_trig::sincos_cr(__ldg(x + i), &s, &c);
        sc[i] = make_float2(s, c);
    }
}

cudaError_t launch_trig_eval(const float* x, float* sincos, long long n, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    const long long blocks = (n + 255) / 256;
    k_trig_eval<<<(unsigned)(blocks < 152 * 64 ? blocks : 152 * 64), 256, 0, s>>>(x, reinterpret_cast<float2*>(sincos), n);
    return cudaGetLastError();
}

// batch kernel variant for (rm_only, layout, pf, separate products)
typedef void (*BatchKernel)(const FilterDev*, int, unsigned, unsigned*);
template <bool SEP>
static BatchKernel batch_kernel_t(bool rm_only, int layout, int pf) {
    if (!rm_only) return k_batch<kAnyKind, 0, 0, SEP>;
    if (pf) {
        if (layout == DT_RUNS) return k_batch<kRmOnly, DT_RUNS, kPrefetch, SEP>;
        if (layout == DT_STEP) return k_batch<kRmOnly, DT_STEP, kPrefetch, SEP>;
        if (layout == DT_U16) return k_batch<kRmOnly, DT_U16, kPrefetch, SEP>;
        if (layout == DT_TILED) return k_batch<kRmOnly, DT_TILED, kPrefetch, SEP>;
        return k_batch<kRmOnly, DT_LINEAR, kPrefetch, SEP>;
    }
    if (layout == DT_RUNS) return k_batch<kRmOnly, DT_RUNS, 0, SEP>;
    if (layout == DT_STEP) return k_batch<kRmOnly, DT_STEP, 0, SEP>;
    if (layout == DT_U16) return k_batch<kRmOnly, DT_U16, 0, SEP>;
    if (layout == DT_TILED) return k_batch<kRmOnly, DT_TILED, 0, SEP>;
    return k_batch<kRmOnly, DT_LINEAR, 0, SEP>;
}
static BatchKernel batch_kernel(bool rm_only, int layout, int pf, bool separate) {
    return separate ? batch_kernel_t<true>(rm_only, layout, pf) : batch_kernel_t<false>(rm_only, layout, pf);
}

cudaError_t launch_fused_staged(const CastParams& p, const SensorDev& sm, const float* ins, const float* angles,
                                const float* obs, double* weights, int n, int na, int chunks,
                                uint16_t* bins, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    if (na <= 0) return launch_fused(p, DT_LINEAR, 0, sm, ins, angles, obs, weights, n, na, 0, 0, s);
    if (chunks <= 0) {   // one block per SM: beams x chunks ~ SM count
        int dev = 0, sms = 152;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        chunks = max(1, sms / na);
    }
    const int P = (n + chunks - 1) / chunks;
    const size_t smem = 1024 + kStagedWindow;
    static std::atomic<unsigned long long> attr{0};
    if (cudaError_t e = ensure_smem_attr(k_bm_cast, (int)smem, attr)) return e;
    dim3 grid(na, (n + P - 1) / P);
    k_bm_cast<<<grid, kStagedThreads, smem, s>>>(p, sm, ins, angles, n, na, P, bins, kStagedWindow / 64);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    const int PB = max(1, min(32, (int)((kTileSmem - (size_t)na * sizeof(uint16_t)) / ((size_t)na * sizeof(double)))));
    const size_t wsmem = (((size_t)PB * na * sizeof(double) + (size_t)na * sizeof(uint16_t)) + 15) & ~(size_t)15;
    e = set_smem(k_bm_weights, wsmem);
    if (e != cudaSuccess) return e;
    k_bm_weights<<<blocks_for(n, PB), 128, wsmem, s>>>(p, sm, obs, bins, n, na, PB, weights);
    return cudaGetLastError();
}

cudaError_t launch_glt_build(const MapDev& map, float mr, unsigned td, const float* cosv, const float* sinv,
                             float limits_div_max, uint16_t* lut, cudaStream_t s) {
    const long long total = (long long)map.W * map.H * td;
    if (total <= 0) return cudaSuccess;
    k_glt_build<<<blocks_for(total, 256), 256, 0, s>>>(map, mr, td, cosv, sinv, limits_div_max, lut, total);
    return cudaGetLastError();
}

cudaError_t launch_cddt_pair(const CastParams& p, float x, float y, float heading, float* out, cudaStream_t s) {
    k_cddt_pair<<<1, 1, 0, s>>>(p, x, y, heading, out);
    return cudaGetLastError();
}

cudaError_t launch_cddt_radial(const CastParams& p, const float* ins, const float* angles, float* outs, int n,
                               int num_rays, int mp, int off, cudaStream_t s) {
    const int A = mp + 1 > off ? mp + 1 : off;
    const long long total = (long long)n * A;
    if (total <= 0 || num_rays <= 0) return cudaSuccess;
    k_cddt_radial<<<blocks_for(total, 256), 256, 0, s>>>(p, ins, angles, outs, n, num_rays, mp, off, A);
    return cudaGetLastError();
}

size_t batch_smem(int block, bool rm_only) {
    return rm_only ? (size_t)((block + 31) / 32) * kBatchSlots * sizeof(RmRay) : 0;
}

cudaError_t batch_occupancy(int block, size_t smem, bool rm_only, int layout, int pf, bool separate,
                            int* blocks_per_sm) {
    BatchKernel k = batch_kernel(rm_only, layout, pf, separate);
    cudaError_t e = set_smem(k, smem);
    if (e != cudaSuccess) return e;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, k, block, smem);
}

cudaError_t launch_batch(const FilterDev* d_filters, int nf, unsigned total_tiles, unsigned* queue, int grid,
                         int block, size_t smem, bool rm_only, int layout, int pf, bool separate,
                         unsigned total_particles, cudaStream_t s) {
    if (total_tiles == 0 || nf == 0) return cudaSuccess;
    BatchKernel k = batch_kernel(rm_only, layout, pf, separate);
    cudaError_t e = set_smem(k, smem);
    if (e != cudaSuccess) return e;
    k_batch_obs_bins<<<nf, 256, 0, s>>>(d_filters, rm_only);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    if (rm_only && total_particles) {
        k_batch_particles<<<blocks_for(total_particles, 256), 256, 0, s>>>(d_filters, nf, total_particles);
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    k<<<grid, block, smem, s>>>(d_filters, nf, total_tiles, queue);
    e = cudaGetLastError();
    if (e != cudaSuccess || !separate || total_particles == 0) return e;
    k_batch_products<<<blocks_for(total_particles, 256), 256, 0, s>>>(d_filters, nf, total_particles);
    return cudaGetLastError();
}

}  // namespace rlc
