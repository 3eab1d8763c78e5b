// Map preprocessing on the device: occupancy bit tiles, the exact Euclidean
// distance transform, the CDDT edge map and the tiled DT copy.
//
// Distance transform: the reference builds it on the CPU with the
// Felzenszwalb-Huttenlocher lower envelope (vendor/distance_transform.h:984-1030,
// called from RangeLib.h:345-373).  k_edt_pass_y/x run the same published
// algorithm, one thread per grid line, with the same float/double operation
// sequence so that every DT value is bit-identical: the intermediate sums
// f[q] + q*q are float (they round above 2^24, which matters on large
// maps), breakpoints are double, and the per-line output is a float.
// Pass 1 runs along y for every x, pass 2 along x for every y.  Maps with
// both sides <= 4096 take k_edt_cols_exact/k_edt_rows_exact instead: the same
// results from a closed form of pass 1 and from pass 2 with its breakpoint
// comparisons decided in integer arithmetic (the argument is given above
// those kernels).
#include "rangelibc.h"
#include "rlc_internal.cuh"

#include <cfloat>
#include <cstdio>
#include <mutex>

namespace rlc {
namespace {

constexpr double kDblMax = 1.7976931348623157e308;

__global__ void k_pack_bits(const uint8_t* __restrict__ occ, int W, int H, int TY, uint64_t* __restrict__ bits) {
    int TX = (W + 7) >> 3;
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)TX * TY) return;
    int tx = (int)(t / TY), ty = (int)(t - (long long)tx * TY);
    uint64_t w = 0;
    for (int i = 0; i < 8; ++i) {
        int x = (tx << 3) + i;
        if (x >= W) break;
        for (int j = 0; j < 8; ++j) {
            int y = (ty << 3) + j;
            if (y >= H) break;
            if (occ[(size_t)x * H + y]) w |= 1ull << ((i << 3) | j);
        }
    }
    bits[t] = w;
}

__device__ __forceinline__ bool occ_bit(const uint64_t* __restrict__ bits, int TY, int x, int y) {
    uint64_t w = bits[(size_t)(x >> 3) * TY + (y >> 3)];
    return (w >> (((x & 7) << 3) | (y & 7))) & 1ull;
}

// One F-H line.  f(q) is the input sample q, out(q, value) stores the
// output; v/z are this line's scratch arrays with a stride of `ld` elements
// between consecutive k (lines interleave so that neighbouring threads touch
// neighbouring words).
template <class In, class Out>
__device__ void fh_line(const In& f, const Out& out, unsigned n, uint32_t* v, double* z, size_t ld) {
    if (n == 0) return;
    if (n == 1) { out(0, f(0)); return; }
    unsigned k = 0;
    v[0] = 0;
    z[0] = -kDblMax;
    z[ld] = kDblMax;
    for (unsigned q = 1; q < n; ++q) {
        double s;
        float fq = __fadd_rn(f(q), __ull2float_rn((unsigned long long)q * q));
        double dq2 = __ull2double_rn(2ull * q);
        ++k;
        do {
            --k;
            unsigned vk = v[(size_t)k * ld];
            float fv = __fadd_rn(f(vk), __ull2float_rn((unsigned long long)vk * vk));
            s = __ddiv_rn(__dsub_rn((double)fq, (double)fv), __dsub_rn(dq2, __ull2double_rn(2ull * vk)));
        } while (s <= z[(size_t)k * ld]);
        ++k;
        v[(size_t)k * ld] = q;
        z[(size_t)k * ld] = s;
        z[(size_t)(k + 1) * ld] = kDblMax;
    }
    k = 0;
    for (unsigned q = 0; q < n; ++q) {
        while (z[(size_t)(k + 1) * ld] < __uint2double_rn(q)) ++k;
        unsigned vk = v[(size_t)k * ld];
        float dq = __fsub_rn(__uint2float_rn(q), __uint2float_rn(vk));
        out(q, __fadd_rn(f(vk), __fmul_rn(dq, dq)));
    }
}

struct OccInput {           // pass 1 input along y for a fixed x
    const uint64_t* bits; int TY; int x;
    __device__ float operator()(unsigned q) const { return occ_bit(bits, TY, x, (int)q) ? 0.0f : FLT_MAX; }
};
struct ColOutput {          // pass 1 output g[x * H + q]
    float* g; size_t base;
    __device__ void operator()(unsigned q, float val) const { g[base + q] = val; }
};
struct RowInput {           // pass 2 input along x for a fixed y: g[q * H + y]
    const float* g; int H; int y;
    __device__ float operator()(unsigned q) const { return g[(size_t)q * H + y]; }
};
struct RowSqrtOutput {      // pass 2 output: sqrt, element_wiseSquareRoot
    float* dt; int H; int y;
    __device__ void operator()(unsigned q, float val) const { dt[(size_t)q * H + y] = __fsqrt_rn(val); }
};

__global__ void k_edt_pass_y(const uint64_t* __restrict__ bits, int W, int H, int TY, float* g,
                             uint32_t* v, double* z) {
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= W) return;
    fh_line(OccInput{bits, TY, x}, ColOutput{g, (size_t)x * H}, (unsigned)H, v + x, z + x, (size_t)W);
}

__global__ void k_edt_pass_x(const float* g, int W, int H, float* dt, uint32_t* v, double* z) {
    int y = blockIdx.x * blockDim.x + threadIdx.x;
    if (y >= H) return;
    fh_line(RowInput{g, H, y}, RowSqrtOutput{dt, H, y}, (unsigned)W, v + y, z + y, (size_t)H);
}

// ---- exact-comparison passes for maps with both sides <= 16384 --------------------------------
//
// For such maps a cheaper computation of the F-H steps above gives the same results bit for bit.
// Every finite key f(q) + q*q (a float sum, as in the reference) is an integer below 2^29, and
// every breakpoint is a quotient a / b of integers with |a| < 2^29 and 2 <= b <= 2 (n - 1) < 2^15,
// computed in double exactly up to the final rounding.  Rounding moves a / b by at most
// 2^-53 |a| / b, while two different quotients a / b and c / d differ by at least 1 / (b d);
// since |a| d + |c| b < 2^45 < 2^53, rounding never reverses or merges two different quotients,
// and equal quotients round alike.  A comparison of rounded breakpoints (s <= z[k],
// z[k + 1] < q) therefore has the outcome of the exact comparison of the quotients, which integer
// cross-multiplication decides.  Comparisons with a FLT_MAX key are evaluated in double exactly
// as the reference does.  The stack holds (v, f(v)) only; breakpoints are recomputed from it.
//  * sides <= 4096, pass 1 (input 0 on occupied cells, FLT_MAX elsewhere): q*q < 2^24 is exact,
//    a breakpoint between two occupied cells p < q is (p + q) / 2, a FLT_MAX parabola is popped
//    by the next occupied cell (their breakpoint is below -FLT_MAX / 8192) or lies beyond the
//    line's end (its breakpoint is above FLT_MAX / 8192), so the envelope picks the nearest
//    occupied cell p and stores (q - p)^2, or FLT_MAX + (q - p)^2 = FLT_MAX in a column without
//    one: a closed form per column (edt_col_exact);
//  * sides <= 4096, pass 2: the stack of each row in shared memory (k_edt_rows_exact);
//  * a side above 4096: q*q rounds, the closed form no longer holds, and both passes run the
//    exact-comparison steps with the stack in global memory (k_edt_cols_fh, k_edt_rows_fh).
constexpr int kEdtExactSide = 4096;           // closed-form pass 1, shared-memory pass 2
constexpr int kEdtIntSide = 16384;            // integer comparisons
constexpr float kEdtExactKey = 536870912.0f;  // 2^29: finite keys are below it

__host__ __device__ __forceinline__ float edt_fadd(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fadd_rn(a, b);
#else
    return a + b;
#endif
}
__host__ __device__ __forceinline__ float edt_fsub(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fsub_rn(a, b);
#else
    return a - b;
#endif
}
__host__ __device__ __forceinline__ float edt_fmul(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fmul_rn(a, b);
#else
    return a * b;
#endif
}
// f(v) + v*v in float, as the reference sums it (v*v < 2^32)
__host__ __device__ __forceinline__ float edt_key(float fv, unsigned v) { return edt_fadd(fv, (float)(v * v)); }
// the reference's breakpoint ((double)kb - (double)ka) / ((double)(2 b) - (double)(2 a))
__host__ __device__ __forceinline__ double edt_isect(float ka, unsigned a, float kb, unsigned b) {
#ifdef __CUDA_ARCH__
    return __ddiv_rn(__dsub_rn((double)kb, (double)ka),
                     __dsub_rn(__ull2double_rn(2ull * b), __ull2double_rn(2ull * a)));
#else
    return ((double)kb - (double)ka) / ((double)(2ull * b) - (double)(2ull * a));
#endif
}
__host__ __device__ __forceinline__ int edt_lsb(unsigned b) {   // b != 0
#ifdef __CUDA_ARCH__
    return __ffs(b) - 1;
#else
    return __builtin_ctz(b);
#endif
}
__host__ __device__ __forceinline__ int edt_msb(unsigned b) {   // b != 0
#ifdef __CUDA_ARCH__
    return 31 - __clz(b);
#else
    return 31 - __builtin_clz(b);
#endif
}

// Pass 1 of one column (H <= 4096).  col[c] is the bit tile of rows 8c..8c+7, the column's byte at
// bit offset sh; nx holds TY + 1 entries of scratch; out[q] receives the squared distance.
__host__ __device__ inline void edt_col_exact(const uint64_t* col, int sh, int H, int TY, uint16_t* nx,
                                              float* out) {
    constexpr unsigned kNone = 0xFFFFu;
    unsigned nxt = kNone;   // first occupied row at or after 8c
    nx[TY] = (uint16_t)kNone;
    for (int c = TY - 1; c >= 0; --c) {
        const unsigned b = (unsigned)(col[c] >> sh) & 0xFFu;
        if (b) nxt = ((unsigned)c << 3) + (unsigned)edt_lsb(b);
        nx[c] = (uint16_t)nxt;
    }
    int prev = -1;          // last occupied row before 8c
    for (int c = 0; c < TY; ++c) {
        const unsigned b = (unsigned)(col[c] >> sh) & 0xFFu;
        const unsigned beyond = nx[c + 1];
        const int base = c << 3, m = H - base < 8 ? H - base : 8;
        for (int j = 0; j < m; ++j) {
            const int q = base + j;
            const unsigned lo = b & ((2u << j) - 1u), hi = b >> j;
            const int p = lo ? base + edt_msb(lo) : prev;
            const unsigned nq = hi ? (unsigned)(q + edt_lsb(hi)) : beyond;
            int d = 0x7FFFFFFF;
            if (p >= 0) d = q - p;
            if (nq != kNone && (int)nq - q < d) d = (int)nq - q;
            out[q] = d == 0x7FFFFFFF ? FLT_MAX : (float)(d * d);
        }
        if (b) prev = base + edt_msb(b);
    }
}

// One line (both sides <= 16384): the reference's F-H steps with the comparisons decided exactly.
// The stack's entry k is (sv[k * ld], sf[k * ld]) -- vertex and its input value -- with room for
// n entries; the top two entries are also kept in registers.
#pragma nv_exec_check_disable
template <class In, class Out>
__host__ __device__ void fh_line_exact(const In& f, const Out& out, unsigned n, uint16_t* sv, float* sf,
                                       size_t ld) {
    if (n == 0) return;
    if (n == 1) { out(0, f(0)); return; }
    unsigned top = 0, vt = 0, vs = 0;   // (vt, kt) entry top, (vs, ks) entry top - 1
    const float f0 = f(0);
    sv[0] = 0;
    sf[0] = f0;
    float kt = edt_key(f0, 0), ks = 0.0f, fnext = f(1);
    for (unsigned q = 1; q < n; ++q) {
        const float fq = fnext;
        if (q + 1 < n) fnext = f(q + 1);
        const float kq = edt_key(fq, q);
        while (top > 0) {   // z[0] = -DBL_MAX: the bottom vertex is never popped
            bool pop;
            if (kq < kEdtExactKey && kt < kEdtExactKey && ks < kEdtExactKey)
                pop = (long long)((int)kq - (int)kt) * (int)(vt - vs) <=
                      (long long)((int)kt - (int)ks) * (int)(q - vt);
            else
                pop = edt_isect(kt, vt, kq, q) <= edt_isect(ks, vs, kt, vt);
            if (!pop) break;
            --top;
            vt = vs;
            kt = ks;
            if (top > 0) {
                vs = sv[(size_t)(top - 1) * ld];
                ks = edt_key(sf[(size_t)(top - 1) * ld], vs);
            }
        }
        ++top;
        sv[(size_t)top * ld] = (uint16_t)q;
        sf[(size_t)top * ld] = fq;
        vs = vt;
        ks = kt;
        vt = q;
        kt = kq;
    }
    unsigned k = 0, vk = sv[0], vn = 0;
    float fk = sf[0], kk = edt_key(fk, vk), fn = 0.0f;
    if (top > 0) {
        vn = sv[ld];
        fn = sf[ld];
    }
    for (unsigned q = 0; q < n; ++q) {
        while (k < top) {   // z[top + 1] = DBL_MAX; (vn, fn) is entry k + 1
            const float kn = edt_key(fn, vn);
            bool adv;
            if (kk < kEdtExactKey && kn < kEdtExactKey)
                adv = (long long)((int)kn - (int)kk) < (long long)q * (long long)(2u * (vn - vk));
            else
                adv = edt_isect(kk, vk, kn, vn) < (double)q;
            if (!adv) break;
            ++k;
            vk = vn;
            fk = fn;
            kk = kn;
            if (k < top) {
                vn = sv[(size_t)(k + 1) * ld];
                fn = sf[(size_t)(k + 1) * ld];
            }
        }
        const float dq = edt_fsub((float)q, (float)vk);
        out(q, edt_fadd(fk, edt_fmul(dq, dq)));
    }
}

// one thread per column; dynamic shared memory: blockDim.x * (TY + 1) uint16
__global__ void k_edt_cols_exact(const uint64_t* __restrict__ bits, int W, int H, int TY, float* __restrict__ g) {
    extern __shared__ uint16_t s_next[];
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= W) return;
    edt_col_exact(bits + (size_t)(x >> 3) * TY, (x & 7) << 3, H, TY, s_next + (size_t)threadIdx.x * (TY + 1),
                  g + (size_t)x * H);
}

// one thread per row; dynamic shared memory: blockDim.x * W * (4 + 2) bytes
__global__ void k_edt_rows_exact(const float* __restrict__ g, int W, int H, float* __restrict__ dt) {
    extern __shared__ __align__(16) unsigned char s_stack[];
    const int y = blockIdx.x * blockDim.x + threadIdx.x;
    if (y >= H) return;
    float* sf = reinterpret_cast<float*>(s_stack) + (size_t)threadIdx.x * W;
    uint16_t* sv = reinterpret_cast<uint16_t*>(reinterpret_cast<float*>(s_stack) + (size_t)blockDim.x * W) +
                   (size_t)threadIdx.x * W;
    fh_line_exact(RowInput{g, H, y}, RowSqrtOutput{dt, H, y}, (unsigned)W, sv, sf, 1);
}

// a side above 4096: one thread per line, the lines' stacks interleaved in global memory
// (entry k of line l at k * lines + l)
__global__ void k_edt_cols_fh(const uint64_t* __restrict__ bits, int W, int H, int TY, float* g, uint16_t* sv,
                              float* sf) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= W) return;
    fh_line_exact(OccInput{bits, TY, x}, ColOutput{g, (size_t)x * H}, (unsigned)H, sv + x, sf + x, (size_t)W);
}

__global__ void k_edt_rows_fh(const float* g, int W, int H, float* dt, uint16_t* sv, float* sf) {
    const int y = blockIdx.x * blockDim.x + threadIdx.x;
    if (y >= H) return;
    fh_line_exact(RowInput{g, H, y}, RowSqrtOutput{dt, H, y}, (unsigned)W, sv + y, sf + y, (size_t)H);
}

__global__ void k_dt_to_tiled(const float* __restrict__ lin, int W, int H, int TY, float* __restrict__ tiled) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    int TX = (W + 7) >> 3;
    if (i >= (long long)TX * TY * 64) return;
    long long tile = i >> 6;
    int within = (int)(i & 63);
    int tx = (int)(tile / TY), ty = (int)(tile - (long long)tx * TY);
    int x = (tx << 3) + (within >> 3), y = (ty << 3) + (within & 7);
    tiled[i] = (x < W && y < H) ? lin[(size_t)x * H + y] : 0.0f;
}

// compact distance transform: uint16 d^2 in 8x8 tiles, 4x4 cells per 32-B sector
__global__ void k_dt_to_u16(const float* __restrict__ lin, int W, int H, int TY, uint16_t* __restrict__ out) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    int TX = (W + 7) >> 3;
    if (i >= (long long)TX * TY * 64) return;
    long long tile = i >> 6;
    int within = (int)(i & 63);
    int sector = within >> 4, cell = within & 15;
    int tx = (int)(tile / TY), ty = (int)(tile - (long long)tx * TY);
    int x = (tx << 3) + ((sector >> 1) << 2) + (cell >> 2);
    int y = (ty << 3) + ((sector & 1) << 2) + (cell & 3);
    uint16_t v = 0xFFFF;
    if (x < W && y < H) {
        // dt = sqrtf(D) for an integer D; D is recovered exactly while D < 2^22
        double d = (double)lin[(size_t)x * H + y];
        double d2 = rint(d * d);
        if (d2 < 65535.0 && __fsqrt_rn((float)d2) == (float)d) v = (uint16_t)d2;
    }
    out[i] = v;
}

// step of the march from each cell, RangeLib.h:957 (t += max(distance * 0.999, 1)); 0 marks an
// occupied cell (distance 0), where the march ends
__global__ void k_dt_to_step(const float* __restrict__ lin, long long n, float* __restrict__ step) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float d = lin[i];
    const float v = __fmul_rn(d, 0.999f);
    step[i] = d <= 0.0f ? 0.0f : (v < 1.0f ? 1.0f : v);
}

// 8-bit squared distance in 8x8 tiles of 64 bytes (x-major within the tile):
// d^2 <= 254 exactly, 255 = "read the float"
__global__ void k_dt_to_u8(const float* __restrict__ lin, int W, int H, int TY, uint8_t* __restrict__ out) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    int TX = (W + 7) >> 3;
    if (i >= (long long)TX * TY * 64) return;
    long long tile = i >> 6;
    int within = (int)(i & 63);
    int tx = (int)(tile / TY), ty = (int)(tile - (long long)tx * TY);
    int x = (tx << 3) + (within >> 3), y = (ty << 3) + (within & 7);
    uint8_t v = 0xFF;
    if (x < W && y < H) {
        double d = (double)lin[(size_t)x * H + y];
        double d2 = rint(d * d);
        if (d2 <= 254.0 && __fsqrt_rn((float)d2) == (float)d) v = (uint8_t)d2;
    }
    out[i] = v;
}

// RangeLib.h:293-312: an occupied cell with any in-grid free 8-neighbour.
__global__ void k_edge_map(const uint64_t* __restrict__ bits, int W, int H, int TY, uint8_t* __restrict__ edge) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)W * H) return;
    int x = (int)(i / H), y = (int)(i - (long long)x * H);
    uint8_t e = 0;
    if (occ_bit(bits, TY, x, y)) {
        for (int dx = -1; dx <= 1 && !e; ++dx)
            for (int dy = -1; dy <= 1; ++dy) {
                if (!dx && !dy) continue;
                int cx = x + dx, cy = y + dy;
                if (cx >= 0 && cy >= 0 && cx < W && cy < H && !occ_bit(bits, TY, cx, cy)) { e = 1; break; }
            }
    }
    edge[i] = e;
}

__global__ void k_unpack_bits(const uint64_t* __restrict__ bits, int W, int H, int TY, uint8_t* __restrict__ occ) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)W * H) return;
    int x = (int)(i / H), y = (int)(i - (long long)x * H);
    occ[i] = occ_bit(bits, TY, x, y) ? 1 : 0;
}

inline unsigned blocks_for(long long n, int b) { return (unsigned)((n + b - 1) / b); }

}  // namespace

cudaError_t launch_pack_bits(const uint8_t* d_occ, int W, int H, uint64_t* d_bits, cudaStream_t s) {
    int TY = (H + 7) >> 3, TX = (W + 7) >> 3;
    long long n = (long long)TX * TY;
    if (n == 0) return cudaSuccess;
    k_pack_bits<<<blocks_for(n, 256), 256, 0, s>>>(d_occ, W, H, TY, d_bits);
    return cudaGetLastError();
}

size_t edt_scratch_bytes(int W, int H) {
    // pass-1 output g (W*H floats) + per-line v (n uint32) and z (n+1 doubles);
    // both passes reuse the same v/z region sized for the larger pass
    size_t g = (size_t)W * H * sizeof(float);
    size_t p1 = (size_t)W * H * sizeof(uint32_t) + (size_t)W * (H + 1) * sizeof(double);
    size_t p2 = (size_t)H * W * sizeof(uint32_t) + (size_t)H * (W + 1) * sizeof(double);
    size_t vz = p1 > p2 ? p1 : p2;
    return ((g + 255) & ~(size_t)255) + vz + 256;
}

cudaError_t launch_edt(const uint64_t* d_bits, int W, int H, int TY, float* d_dt, void* scratch,
                       size_t scratch_bytes, cudaStream_t s) {
    if (W <= 0 || H <= 0) return cudaSuccess;
    if (scratch_bytes < edt_scratch_bytes(W, H)) return cudaErrorInvalidValue;
    char* base = static_cast<char*>(scratch);
    float* g = reinterpret_cast<float*>(base);
    if (W <= kEdtExactSide && H <= kEdtExactSide) {
        k_edt_cols_exact<<<blocks_for(W, 32), 32, 32 * (TY + 1) * sizeof(uint16_t), s>>>(d_bits, W, H, TY, g);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        // rows per block: the stack's shared memory, and about one block per SM of a 152-SM part
        constexpr int kSmemCap = 227 * 1024;
        const int per_line = W * (int)(sizeof(float) + sizeof(uint16_t));
        int lines = (H + 151) / 152;
        lines = lines < kSmemCap / per_line ? lines : kSmemCap / per_line;
        lines = lines < 32 ? (lines > 0 ? lines : 1) : 32;
        static std::atomic<unsigned long long> attr_done{0};
        e = ensure_smem_attr(k_edt_rows_exact, kSmemCap, attr_done);
        if (e != cudaSuccess) return e;
        k_edt_rows_exact<<<blocks_for(H, lines), lines, (size_t)lines * per_line, s>>>(g, W, H, d_dt);
        return cudaGetLastError();
    }
    size_t goff = ((size_t)W * H * sizeof(float) + 255) & ~(size_t)255;
    if (W <= kEdtIntSide && H <= kEdtIntSide) {   // stacks: W * H floats, then W * H uint16 (either pass)
        float* sf = reinterpret_cast<float*>(base + goff);
        uint16_t* sv = reinterpret_cast<uint16_t*>(base + goff + (size_t)W * H * sizeof(float));
        k_edt_cols_fh<<<blocks_for(W, 32), 32, 0, s>>>(d_bits, W, H, TY, g, sv, sf);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        k_edt_rows_fh<<<blocks_for(H, 32), 32, 0, s>>>(g, W, H, d_dt, sv, sf);
        return cudaGetLastError();
    }
    // per pass: z (n+1 doubles per line) first, then v (n uint32 per line)
    double* z1 = reinterpret_cast<double*>(base + goff);
    uint32_t* v1 = reinterpret_cast<uint32_t*>(base + goff + (size_t)W * (H + 1) * sizeof(double));
    k_edt_pass_y<<<blocks_for(W, 64), 64, 0, s>>>(d_bits, W, H, TY, g, v1, z1);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    double* z2 = reinterpret_cast<double*>(base + goff);
    uint32_t* v2 = reinterpret_cast<uint32_t*>(base + goff + (size_t)H * (W + 1) * sizeof(double));
    k_edt_pass_x<<<blocks_for(H, 64), 64, 0, s>>>(g, W, H, d_dt, v2, z2);
    return cudaGetLastError();
}

cudaError_t launch_dt_to_tiled(const float* d_lin, int W, int H, float* d_tiled, cudaStream_t s) {
    int TY = (H + 7) >> 3, TX = (W + 7) >> 3;
    long long n = (long long)TX * TY * 64;
    if (n == 0) return cudaSuccess;
    k_dt_to_tiled<<<blocks_for(n, 256), 256, 0, s>>>(d_lin, W, H, TY, d_tiled);
    return cudaGetLastError();
}

cudaError_t launch_dt_to_u16(const float* d_lin, int W, int H, uint16_t* d_u16, cudaStream_t s) {
    int TY = (H + 7) >> 3, TX = (W + 7) >> 3;
    long long n = (long long)TX * TY * 64;
    if (n == 0) return cudaSuccess;
    k_dt_to_u16<<<blocks_for(n, 256), 256, 0, s>>>(d_lin, W, H, TY, d_u16);
    return cudaGetLastError();
}

cudaError_t launch_dt_to_step(const float* d_lin, int W, int H, float* d_step, cudaStream_t s) {
    const long long n = (long long)W * H;
    if (n == 0) return cudaSuccess;
    k_dt_to_step<<<blocks_for(n, 256), 256, 0, s>>>(d_lin, n, d_step);
    return cudaGetLastError();
}

// Equal-step runs along y: one thread per column x walks it both ways; bits 0-7 of runs[x * H + y]
// count the cells y + 1, y + 2, ... whose step equals the step of (x, y), bits 8-15 the cells
// y - 1, y - 2, ... (at most 255 each); bits 16-31 are cleared for the x pass.
__global__ void k_step_runs_y(const float* __restrict__ step, int W, int H, uint32_t* __restrict__ runs) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= W) return;
    const float* col = step + (size_t)x * H;
    uint32_t* out = runs + (size_t)x * H;
    unsigned run = 0;
    for (int y = 1; y < H; ++y) {   // -y: run ending just below y
        run = col[y - 1] == col[y] ? min(run + 1u, 255u) : 0u;
        out[y] = run << 8;
    }
    out[0] = 0u;
    run = 0;
    for (int y = H - 2; y >= 0; --y) {   // +y
        run = col[y + 1] == col[y] ? min(run + 1u, 255u) : 0u;
        out[y] |= run;
    }
}

// the same along x, one thread per row y: bits 16-23 (+x) and 24-31 (-x)
__global__ void k_step_runs_x(const float* __restrict__ step, int W, int H, uint32_t* __restrict__ runs) {
    const int y = blockIdx.x * blockDim.x + threadIdx.x;
    if (y >= H) return;
    unsigned run = 0;
    for (int x = 1; x < W; ++x) {
        const size_t i = (size_t)x * H + y;
        run = step[i - H] == step[i] ? min(run + 1u, 255u) : 0u;
        runs[i] |= run << 24;
    }
    run = 0;
    for (int x = W - 2; x >= 0; --x) {
        const size_t i = (size_t)x * H + y;
        run = step[i + H] == step[i] ? min(run + 1u, 255u) : 0u;
        runs[i] |= run << 16;
    }
}

cudaError_t launch_step_runs(const float* d_step, int W, int H, uint32_t* d_runs, cudaStream_t s) {
    if ((long long)W * H == 0) return cudaSuccess;
    k_step_runs_y<<<blocks_for(W, 128), 128, 0, s>>>(d_step, W, H, d_runs);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_step_runs_x<<<blocks_for(H, 128), 128, 0, s>>>(d_step, W, H, d_runs);
    return cudaGetLastError();
}

cudaError_t launch_dt_to_u8(const float* d_lin, int W, int H, uint8_t* d_u8, cudaStream_t s) {
    int TY = (H + 7) >> 3, TX = (W + 7) >> 3;
    long long n = (long long)TX * TY * 64;
    if (n == 0) return cudaSuccess;
    k_dt_to_u8<<<blocks_for(n, 256), 256, 0, s>>>(d_lin, W, H, TY, d_u8);
    return cudaGetLastError();
}

cudaError_t launch_edge_map(const uint64_t* d_bits, int W, int H, int TY, uint8_t* d_edge, cudaStream_t s) {
    long long n = (long long)W * H;
    if (n == 0) return cudaSuccess;
    k_edge_map<<<blocks_for(n, 256), 256, 0, s>>>(d_bits, W, H, TY, d_edge);
    return cudaGetLastError();
}

cudaError_t launch_unpack_bits(const uint64_t* d_bits, int W, int H, int TY, uint8_t* d_occ, cudaStream_t s) {
    long long n = (long long)W * H;
    if (n == 0) return cudaSuccess;
    k_unpack_bits<<<blocks_for(n, 256), 256, 0, s>>>(d_bits, W, H, TY, d_occ);
    return cudaGetLastError();
}

}  // namespace rlc

// ===========================================================================
// rlc_distance_transform_noalloc: the distance transform for callers that
// cannot allocate device memory.
//
// Some callers may not call cudaMalloc at all: real-time loops (a robot's
// localisation node) that forbid allocation after start-up, and hosts whose
// device memory belongs to another allocator (a framework's caching
// allocator, a fixed pool handed out by an embedding application).  This
// entry point computes the same distance transform as
// rlc_map_distance_transform from a caller-owned device occupancy grid into
// a caller-owned device output, and keeps every intermediate (the packed
// occupancy bits, the first-pass output and the per-line envelope arrays) in
// one file-scope device array of fixed size, so it allocates nothing.
//
// * The array holds RLC_NOALLOC_SCRATCH_BYTES (~16.2 MiB) on every GPU that
//   loads this library, until the process exits.
// * Maps are limited to RLC_NOALLOC_MAX_CELLS cells with sides of at most
//   RLC_NOALLOC_MAX_SIDE; larger maps are rejected with RLC_ERR_ARG.
// * The first call on a device looks up the array's device address there
//   (cudaGetSymbolAddress, with that device current) and caches it; make
//   that first call before any stream capture.  The cached address lives as
//   long as the device's primary context: after cudaDeviceReset the library
//   has to be unloaded and loaded again before this entry point is used.
// * All calls share the array and it keeps the last call's contents.  No
//   word of it needs to start at zero (each is written before it is read),
//   but calls that overlap on the GPU -- on different streams, or from
//   different host threads -- race on it and corrupt each other's results.
// ===========================================================================
namespace rlc {
namespace {

constexpr size_t align_up(size_t b) { return (b + 255) & ~(size_t)255; }
constexpr size_t kNoAllocMaxCells = RLC_NOALLOC_MAX_CELLS;
constexpr size_t kNoAllocMaxSide = RLC_NOALLOC_MAX_SIDE;
// packed bits: ceil(W/8) * ceil(H/8) words <= cells/64 + (W + H)/8 + 1
constexpr size_t kNoAllocBitsBytes = align_up((kNoAllocMaxCells / 64 + 2 * kNoAllocMaxSide / 8 + 1) * 8);
constexpr size_t kNoAllocScratchBytes = kNoAllocBitsBytes + edt_scratch_bound(kNoAllocMaxCells, kNoAllocMaxSide);
static_assert(kNoAllocScratchBytes == RLC_NOALLOC_SCRATCH_BYTES, "rangelibc.h states the scratch size");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
void* g_noalloc_addr[kMaxDevices] = {};

// device address of g_noalloc_scratch on the current device (looked up once per device)
int noalloc_scratch(void** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    char msg[256];
    if (e != cudaSuccess) {
        snprintf(msg, sizeof(msg), "rlc_distance_transform_noalloc: %s", cudaGetErrorString(e));
        return set_last_error(RLC_ERR_CUDA, msg);
    }
    if (dev < 0 || dev >= kMaxDevices) return set_last_error(RLC_ERR_CUDA, "rlc_distance_transform_noalloc: device ordinal out of range");
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            snprintf(msg, sizeof(msg), "rlc_distance_transform_noalloc: scratch address: %s",
                     cudaGetErrorString(e));
            return set_last_error(RLC_ERR_CUDA, msg);
        }
        g_noalloc_addr[dev] = p;
    }
    *out = g_noalloc_addr[dev];
    return RLC_OK;
}

// device memory of the current device, or managed memory; memory of another device is refused
// (without peer access the kernels here would fault on it)
bool is_device_pointer(const void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    if (a.type == cudaMemoryTypeManaged) return true;
    if (a.type != cudaMemoryTypeDevice) return false;
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.device == dev;
}

}  // namespace
}  // namespace rlc

extern "C" int rlc_distance_transform_noalloc(const uint8_t* d_occ, int width, int height, float* d_dt,
                                              void* stream) {
    using namespace rlc;
    char msg[256];
    if (!d_occ || !d_dt) return set_last_error(RLC_ERR_ARG, "rlc_distance_transform_noalloc: null pointer");
    if (width <= 0 || height <= 0) return set_last_error(RLC_ERR_ARG, "rlc_distance_transform_noalloc: sizes must be positive");
    if ((size_t)width > kNoAllocMaxSide || (size_t)height > kNoAllocMaxSide ||
        (size_t)width * (size_t)height > kNoAllocMaxCells) {
        snprintf(msg, sizeof(msg),
                 "rlc_distance_transform_noalloc: a %dx%d map exceeds the fixed scratch (at most %zu cells and "
                 "%zu per side); use rlc_map_create + rlc_map_distance_transform",
                 width, height, kNoAllocMaxCells, kNoAllocMaxSide);
        return set_last_error(RLC_ERR_ARG, msg);
    }
    if (!is_device_pointer(d_occ) || !is_device_pointer(d_dt))
        return set_last_error(RLC_ERR_ARG, "rlc_distance_transform_noalloc: d_occ and d_dt must be device memory of the current device");
    void* base = nullptr;
    if (int rc = noalloc_scratch(&base)) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    uint64_t* bits = static_cast<uint64_t*>(base);
    void* edt_scratch = static_cast<char*>(base) + kNoAllocBitsBytes;
    const int TY = (height + 7) >> 3;
    cudaError_t e = launch_pack_bits(d_occ, width, height, bits, s);
    if (e == cudaSuccess)
        e = launch_edt(bits, width, height, TY, d_dt, edt_scratch, kNoAllocScratchBytes - kNoAllocBitsBytes, s);
    if (e != cudaSuccess) {
        snprintf(msg, sizeof(msg), "rlc_distance_transform_noalloc: %s", cudaGetErrorString(e));
        return set_last_error(RLC_ERR_CUDA, msg);
    }
    return RLC_OK;
}
