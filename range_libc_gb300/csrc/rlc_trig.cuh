// Correctly rounded float sine and cosine for the per-ray headings of ray
// marching and Bresenham's line.
//
// The reference computes each ray's cosf/sinf with the host C library
// (RangeLib.h:700-702, 930-931), and a ray's hit cell can change with the
// last bit of either.  No fixed rule reproduces every libm (glibc's float
// sine and cosine are themselves not correctly rounded on about 0.1 % of
// arguments); the rule here is the one every accurate libm agrees with
// almost everywhere: the float nearest to the exact sin(x) and cos(x).
//
// Method (written for this library):
//  1. |x| < 2^-12: sin = x and cos = 1 are the correctly rounded values.
//  2. |x| < 4096: j = rint(x * 2/pi) and r = x - j * pi/2 as a float pair,
//     with pi/2 split into four floats (Cody-Waite): j * C0 and j * C1 are
//     formed exactly (two-product by FMA), x - fl(j * C0) is exact
//     (Sterbenz), and the tail terms are summed in float.  |r| <= pi/4 + 2^-11.
//  3. k = rint(256 r), u = r - k/256 (|u| <= 2^-9, renormalised float pair);
//     sin(r) = S_k cos(u) + C_k sin(u), cos(r) = C_k cos(u) - S_k sin(u),
//     with S_k, C_k = sin, cos(k/256) as float pairs (rlc_trig_table.h,
//     computed with mpmath) and short Taylor series for sin(u) and cos(u)
//     (the first omitted terms are below 2^-54 relative).  The largest
//     products are formed exactly, the small corrections in float.
//  4. The result is a float pair (h, l) within 2^-42 of the exact value
//     (relative), so h is the correctly rounded value unless the exact value
//     may lie across a rounding midpoint of h: the code checks
//     |l| + 2^-40 |h| < (half the spacing of floats at h), and
//  5. otherwise (about 1 argument in 2^15, |x| >= 4096, a reduced argument
//     below 2^-16 after a reduction, NaN, infinities) rounds the double
//     precision sin and cos, whose error (a few units in the 53rd bit) can
//     misround only arguments within ~2^-50 of a midpoint.
//  6. sincos_diff: for a ray heading h = fl(th - a) whose th and a have float
//     pairs of their sin and cos (sincos_pairs: the pairs of step 4 before
//     rounding), the angle-difference formulas with an exact correction for
//     the rounding of th - a give pairs within 2^-40.2 of sin h and cos h; a
//     rounding check against 2^-39 (absolute) certifies their high parts as
//     the values of sincos_cr, else the caller computes them directly.
//
// Every operation is written out (no contraction: the library is compiled
// with -fmad=false and host checks with -ffp-contract=off), so the host and
// the device compute the same bits; tests/cpp/trig_check.cpp compares the
// host build against the exact values and the device kernels against it.
#pragma once

#include <math.h>
#include <stdint.h>
#include <string.h>

#include "rlc_trig_table.h"

#if defined(__CUDACC__)
#define RLC_TRIG_HD __host__ __device__ __forceinline__
#else
#define RLC_TRIG_HD static inline
#endif

namespace rlc_trig {

struct F2 {
    float h, l;
};

struct Row {
    float sh, sl, ch, cl;
};

#if defined(__CUDACC__)
__device__ __align__(16) const Row kTableDev[RLC_TRIG_KMAX + 1] = {RLC_TRIG_TABLE_ROWS};
#endif
static const Row kTableHost[RLC_TRIG_KMAX + 1] = {RLC_TRIG_TABLE_ROWS};

RLC_TRIG_HD uint32_t bits_of(float f) {
#if defined(__CUDA_ARCH__)
    return __float_as_uint(f);
#else
    uint32_t u;
    memcpy(&u, &f, 4);
    return u;
#endif
}

RLC_TRIG_HD float float_of(uint32_t u) {
#if defined(__CUDA_ARCH__)
    return __uint_as_float(u);
#else
    float f;
    memcpy(&f, &u, 4);
    return f;
#endif
}

RLC_TRIG_HD Row row(int k) {
#if defined(__CUDA_ARCH__)
    const float4 v = __ldg(reinterpret_cast<const float4*>(kTableDev) + k);
    return Row{v.x, v.y, v.z, v.w};
#else
    return kTableHost[k];
#endif
}

// s + e = a + b exactly
RLC_TRIG_HD F2 two_sum(float a, float b) {
    const float s = a + b;
    const float bb = s - a;
    const float e = (a - (s - bb)) + (b - bb);
    return F2{s, e};
}

// s + e = a + b exactly, given a == 0 or exponent(a) >= exponent(b)
RLC_TRIG_HD F2 fast_two_sum(float a, float b) {
    const float s = a + b;
    return F2{s, b - (s - a)};
}

// p + e = a * b exactly (no underflow here)
RLC_TRIG_HD F2 two_prod(float a, float b) {
    const float p = a * b;
    return F2{p, fmaf(a, b, -p)};
}

// true when h is the correctly rounded value of every number within 2^-40 |h| of h + l
// (h normal, |l| <= half an ulp of h)
RLC_TRIG_HD bool rounds_safely(F2 v) {
    const float ah = fabsf(v.h);
    const uint32_t b = bits_of(ah);
    const float ulp = float_of(b & 0x7f800000u) * 0x1p-23f;
    const float half = (b & 0x007fffffu) ? ulp * 0.5f : ulp * 0.25f;   // below a power of two: a quarter
    return fabsf(v.l) + ah * 0x1p-40f < half;
}

// Steps 2 and 3 for 2^-12 <= |x| < 4096: float pairs of sin and cos of the reduced argument
// r = x - j pi/2, and j mod 4; false where the reduction's relative error grows.
RLC_TRIG_HD bool sincos_reduced(float x, F2* sr_out, F2* cr_out, int* q_out) {
    // 2. reduction
    const float j = rintf(x * RLC_TRIG_TWO_OVER_PI);
    const F2 p0 = two_prod(j, RLC_TRIG_C0);
    const float t = x - p0.h;   // exact
    const F2 p1 = two_prod(j, RLC_TRIG_C1);
    const F2 a = two_sum(t, -p0.l);
    const F2 b = two_sum(a.h, -p1.h);
    const float tail = fmaf(j, RLC_TRIG_C3, fmaf(j, RLC_TRIG_C2, p1.l));
    const float rest = (a.l + b.l) - tail;
    const F2 r = fast_two_sum(b.h, rest);
    if (j != 0.0f && fabsf(r.h) < 0x1p-16f) return false;   // the reduction's relative error grows
    // 3. r = k/256 + u
    const float kf = rintf(r.h * 256.0f);
    const int k = (int)kf;
    const float uh = r.h - kf * 0x1p-8f;   // exact
    const F2 u = fast_two_sum(uh, r.l);
    const F2 u2 = two_prod(u.h, u.h);
    const float u2t = fmaf(2.0f * u.h, u.l, u2.l);                    // u^2 = u2.h + u2t (+ u.l^2)
    const float q1 = -0.5f * u2.h;                                     // cos u = 1 + q1 + q2
    const float q2 = fmaf(u2.h * u2.h, 1.0f / 24.0f, -0.5f * u2t);
    const float P = u2.h * fmaf(u2.h, 1.0f / 120.0f, -1.0f / 6.0f);   // sin u = u + u P
    const float su_l = fmaf(u.h, P, u.l);                              // sin u = u.h + su_l
    Row T = row(k < 0 ? -k : k);
    if (k < 0) {
        T.sh = -T.sh;
        T.sl = -T.sl;
    }
    // sin r = S + S q1 + S q2 + C u.h + C su_l
    const F2 ms = two_prod(T.ch, u.h);
    const F2 as = two_sum(T.sh, ms.h);
    float cs = T.sl + as.l + ms.l;
    cs = fmaf(T.cl, u.h, cs);
    cs = fmaf(T.ch, su_l, cs);
    cs = fmaf(T.sh, q2, cs);
    cs = fmaf(T.sl, q1, cs);
    cs = fmaf(T.sh, q1, cs);
    const F2 sr = fast_two_sum(as.h, cs);
    // cos r = C + C q1 + C q2 - S u.h - S su_l
    const F2 mc = two_prod(T.sh, u.h);
    const F2 ac = two_sum(T.ch, -mc.h);
    float cc = T.cl + ac.l - mc.l;
    cc = fmaf(-T.sl, u.h, cc);
    cc = fmaf(-T.sh, su_l, cc);
    cc = fmaf(T.ch, q2, cc);
    cc = fmaf(T.cl, q1, cc);
    cc = fmaf(T.ch, q1, cc);
    const F2 cr = fast_two_sum(ac.h, cc);
    *sr_out = sr;
    *cr_out = cr;
    *q_out = (int)j & 3;
    return true;
}

// Fast path: returns false where the double-precision fallback must decide.
RLC_TRIG_HD bool sincos_fast(float x, float* sp, float* cp) {
    const float ax = fabsf(x);
    if (!(ax < 4096.0f)) return false;   // also NaN and infinities
    if (ax < 0x1p-12f) {
        *sp = x;
        *cp = 1.0f;
        return true;
    }
    F2 sr, cr;
    int q;
    if (!sincos_reduced(x, &sr, &cr, &q)) return false;
    if (!rounds_safely(sr) || !rounds_safely(cr)) return false;
    const float s = sr.h, c = cr.h;
    *sp = (q == 0) ? s : (q == 1) ? c : (q == 2) ? -s : -c;
    *cp = (q == 0) ? c : (q == 1) ? -s : (q == 2) ? -c : s;
    return true;
}

// sin(x) and cos(x) as float pairs within 2^-42 of the exact values (relative): the fast path's
// values before their rounding, turned to x's quadrant.  False for |x| < 2^-12, |x| >= 4096,
// NaN, infinities and where the reduction's relative error grows.
RLC_TRIG_HD bool sincos_pairs(float x, F2* sp, F2* cp) {
    const float ax = fabsf(x);
    if (!(ax < 4096.0f) || ax < 0x1p-12f) return false;
    F2 sr, cr;
    int q;
    if (!sincos_reduced(x, &sr, &cr, &q)) return false;
    const F2 ns{-sr.h, -sr.l}, nc{-cr.h, -cr.l};
    *sp = (q == 0) ? sr : (q == 1) ? cr : (q == 2) ? ns : nc;
    *cp = (q == 0) ? cr : (q == 1) ? ns : (q == 2) ? nc : sr;
    return true;
}

// true when h is the correctly rounded value of every number within 2^-39 of h + l (absolute;
// h normal, |l| <= half an ulp of h)
RLC_TRIG_HD bool rounds_safely_abs(F2 v) {
    const float ah = fabsf(v.h);
    const uint32_t b = bits_of(ah);
    const float ulp = float_of(b & 0x7f800000u) * 0x1p-23f;
    const float half = (b & 0x007fffffu) ? ulp * 0.5f : ulp * 0.25f;   // below a power of two: a quarter
    return fabsf(v.l) + 0x1p-39f < half;
}

// The correctly rounded sin h and cos h of h = fl(th - a) from float pairs of sin and cos of th
// (ps, pc) and of a (bs, bc), each within 2^-42 of its exact value (relative; sincos_pairs), or
// false where the caller must compute them directly.  th - a = h + e exactly (two_sum), and
//   sin h = sin(th - a) cos e - cos(th - a) sin e,   cos h = cos(th - a) cos e + sin(th - a) sin e,
//   sin(th - a) = ps bc - pc bs,   cos(th - a) = pc bc + ps bs.
// The products of the high parts are formed exactly, every other term (the products' errors, the
// cross terms with the low parts, -e cos(th - a) and e sin(th - a)) is summed in one float.  For
// |e| <= 2^-21 the results lie within 2^-40.2 of sin h and cos h: 2^-41 from the four inputs
// (|sin th cos a| + |cos th sin a| <= 1), 2^-43 for the dropped e^2 / 2 terms, about 2^-42.2 for
// the float sums of the low terms and the e terms, below 2^-47 for the dropped products of low
// parts; rounds_safely_abs then allows for 2^-39.
RLC_TRIG_HD bool sincos_diff(float th, float a, F2 ps, F2 pc, F2 bs, F2 bc, float* sp, float* cp) {
    const F2 d = two_sum(th, -a);   // d.h = fl(th - a) = h
    const float e = d.l;
    if (!(fabsf(e) <= 0x1p-21f)) return false;
    const F2 p1 = two_prod(ps.h, bc.h), p2 = two_prod(pc.h, bs.h);
    const F2 p3 = two_prod(pc.h, bc.h), p4 = two_prod(ps.h, bs.h);
    const F2 s0 = two_sum(p1.h, -p2.h), c0 = two_sum(p3.h, p4.h);
    float sl = fmaf(ps.h, bc.l, fmaf(ps.l, bc.h, p1.l - p2.l));
    sl = fmaf(-pc.h, bs.l, fmaf(-pc.l, bs.h, sl));
    float cl = fmaf(pc.h, bc.l, fmaf(pc.l, bc.h, p3.l + p4.l));
    cl = fmaf(ps.h, bs.l, fmaf(ps.l, bs.h, cl));
    sl = fmaf(-e, c0.h, s0.l + sl);
    cl = fmaf(e, s0.h, c0.l + cl);
    const F2 S = two_sum(s0.h, sl), C = two_sum(c0.h, cl);
    if (!rounds_safely_abs(S) || !rounds_safely_abs(C)) return false;
    *sp = S.h;
    *cp = C.h;
    return true;
}

// the double-precision fallback, kept out of line on the device (it is rarely taken)
#if defined(__CUDACC__)
static __device__ __noinline__ float2 sincos_slow_dev(float x) {
    double sd, cd;
    sincos((double)x, &sd, &cd);
    return make_float2((float)sd, (float)cd);
}
#endif

// The float nearest to sin(x) and to cos(x).
RLC_TRIG_HD void sincos_cr(float x, float* sp, float* cp) {
    if (sincos_fast(x, sp, cp)) return;
#if defined(__CUDA_ARCH__)
    const float2 v = sincos_slow_dev(x);
    *sp = v.x;
    *cp = v.y;
#else
    const double xd = (double)x;
    *sp = (float)sin(xd);
    *cp = (float)cos(xd);
#endif
}

}  // namespace rlc_trig
