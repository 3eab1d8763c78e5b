// Map preprocessing on the device: occupancy bit tiles, the exact Euclidean
// distance transform, the CDDT edge map and the tiled DT copy.
//
// Distance transform: the reference builds it on the CPU with the
// Felzenszwalb-Huttenlocher lower envelope (vendor/distance_transform.h:984-1030,
// called from RangeLib.h:345-373).  The kernels below run the same published
// algorithm, one thread per grid line, with the same float/double operation
// sequence so that every DT value is bit-identical: the intermediate sums
// f[q] + q*q are float (they round above 2^24, which matters on 4096^2
// maps), breakpoints are double, and the per-line output is a float.
// Pass 1 runs along y for every x, pass 2 along x for every y.
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
    size_t goff = ((size_t)W * H * sizeof(float) + 255) & ~(size_t)255;
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
//   that first call before any stream capture.
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

bool is_device_pointer(const void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
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
        return set_last_error(RLC_ERR_ARG, "rlc_distance_transform_noalloc: d_occ and d_dt must be device memory");
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
