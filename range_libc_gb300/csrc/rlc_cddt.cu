// CDDT (compressed directional distance transform) table, built and pruned
// on the device, plus the scan primitive it uses.
//
// The table follows the reference's construction (RangeLib.h:974-1159):
// for every edge pixel and every slice a < td/2, the pixel centre is
// projected into the slice's rotated frame and its x coordinate is appended
// to each bin its y extent covers; every bin is then sorted and
// de-duplicated.  Prune (RangeLib.h:1176-1283) replays a query from every
// free cell centre of every slice and keeps only the zero points a query can
// return.  Here those steps are: an edge map, a count pass and a fill pass
// (one thread per edge pixel and slice), an exclusive scan to CSR offsets,
// a per-bin bitonic sort in shared memory with de-duplication, and a final
// compaction; prune marks used entries with one thread per (cell, slice)
// and compacts with the same scan.
//
// Device layout: slice a owns bins [slice_base[a], slice_base[a+1]); bin b
// owns zeros [bin_start[b], bin_start[b+1]).  All offsets are uint32.
#include "rlc_internal.cuh"

#include <cstdio>
#include <vector>

namespace rlc {
namespace {

constexpr double kEps = 0.00001;   // RangeLib.h:60 _EPSILON
constexpr int kBinarySearchThreshold = 64;

inline unsigned blocks_for(long long n, int b) { return (unsigned)((n + b - 1) / b); }

// ------------------------------------------------------------------- scan
constexpr int kScanThreads = 512;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

struct OpSum {
    typedef uint32_t T;
    static __device__ __forceinline__ T id() { return 0u; }
    static __device__ __forceinline__ T op(T a, T b) { return a + b; }
};
struct OpMax {
    typedef int T;
    static __device__ __forceinline__ T id() { return -2147483647 - 1; }
    static __device__ __forceinline__ T op(T a, T b) { return a > b ? a : b; }
};

// block-wide scan of one value per thread: returns the exclusive prefix,
// `total` gets the reduction over the block
template <class Op>
__device__ __forceinline__ typename Op::T block_scan(typename Op::T v, typename Op::T* warp_vals,
                                                     typename Op::T& total) {
    typedef typename Op::T T;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    T x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        T y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x = Op::op(y, x);
    }
    T excl_in_warp = __shfl_up_sync(0xffffffffu, x, 1);
    if (lane == 0) excl_in_warp = Op::id();
    if (lane == 31) warp_vals[wid] = x;
    __syncthreads();
    if (wid == 0) {
        const int nw = blockDim.x >> 5;
        T w = lane < nw ? warp_vals[lane] : Op::id();
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            T y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w = Op::op(y, w);
        }
        if (lane < nw) warp_vals[lane] = w;
    }
    __syncthreads();
    total = warp_vals[(blockDim.x >> 5) - 1];
    T excl = wid > 0 ? Op::op(warp_vals[wid - 1], excl_in_warp) : excl_in_warp;
    __syncthreads();
    return excl;
}

template <class Op>
__global__ void __launch_bounds__(kScanThreads) k_tile_reduce(const typename Op::T* __restrict__ in, size_t n,
                                                              typename Op::T* __restrict__ sums) {
    __shared__ typename Op::T ws[32];
    size_t base = (size_t)blockIdx.x * kScanTile + (size_t)threadIdx.x * kScanItems;
    typename Op::T s = Op::id();
#pragma unroll
    for (int i = 0; i < kScanItems; ++i)
        if (base + i < n) s = Op::op(s, in[base + i]);
    typename Op::T total;
    block_scan<Op>(s, ws, total);
    if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

// single block: exclusive scan of the tile reductions in place; sums[ntiles] = total
template <class Op>
__global__ void __launch_bounds__(kScanThreads) k_scan_partials(typename Op::T* sums, size_t ntiles) {
    __shared__ typename Op::T ws[32];
    typename Op::T carry = Op::id();
    for (size_t base = 0; base < ntiles; base += kScanThreads) {
        size_t i = base + threadIdx.x;
        typename Op::T v = i < ntiles ? sums[i] : Op::id();
        typename Op::T total;
        typename Op::T e = block_scan<Op>(v, ws, total);
        if (i < ntiles) sums[i] = Op::op(carry, e);
        carry = Op::op(carry, total);
    }
    if (threadIdx.x == 0) sums[ntiles] = carry;
}

// INCLUSIVE = false: out[i] = op(in[0..i-1]) and out[n] = total; true: out[i] = op(in[0..i])
template <class Op, bool INCLUSIVE>
__global__ void __launch_bounds__(kScanThreads) k_scan_tiles(const typename Op::T* __restrict__ in, size_t n,
                                                             const typename Op::T* __restrict__ sums,
                                                             typename Op::T* __restrict__ out, size_t ntiles) {
    typedef typename Op::T T;
    __shared__ T ws[32];
    size_t base = (size_t)blockIdx.x * kScanTile + (size_t)threadIdx.x * kScanItems;
    T v[kScanItems];
    T s = Op::id();
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        v[i] = base + i < n ? in[base + i] : Op::id();
        s = Op::op(s, v[i]);
    }
    T total;
    T run = Op::op(sums[blockIdx.x], block_scan<Op>(s, ws, total));
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        if (INCLUSIVE) run = Op::op(run, v[i]);
        if (base + i < n) out[base + i] = run;
        if (!INCLUSIVE) run = Op::op(run, v[i]);
    }
    if (!INCLUSIVE && blockIdx.x == 0 && threadIdx.x == 0) out[n] = sums[ntiles];
}

// ------------------------------------------------------------ construction
__device__ __forceinline__ bool occ_bit(const uint64_t* __restrict__ bits, int TY, int x, int y) {
    uint64_t w = __ldg(bits + (size_t)(x >> 3) * TY + (y >> 3));
    return (w >> (((x & 7) << 3) | (y & 7))) & 1ull;
}

struct SliceGeom {
    const int* widths;
    const float* trans;
    const float* cosv;
    const float* sinv;
    const uint32_t* slice_base;
};

// RangeLib.h:1086-1103: projection of a pixel centre into slice a.
__device__ __forceinline__ void project_pixel(const SliceGeom& g, int a, int x, int y, float& lcx, int& lower,
                                              int& upper) {
    const float ca = __ldg(g.cosv + a), sa = __ldg(g.sinv + a);
    const float half = __fmul_rn(__fadd_rn(fabsf(sa), fabsf(ca)), 0.5f);   // (|s|+|c|) / 2.0, exact halving
    const float px = __int2float_rn(x) + 0.5f, py = __int2float_rn(y) + 0.5f;   // exact for grids < 2^23
    lcx = __fsub_rn(__fmul_rn(px, ca), __fmul_rn(py, sa));
    const float lcy = __fadd_rn(__fadd_rn(__fmul_rn(px, sa), __fmul_rn(py, ca)), __ldg(g.trans + a));
    upper = __double2int_rz(__dsub_rn((double)__fadd_rn(lcy, half), kEps));
    lower = __double2int_rz(__dadd_rn((double)__fsub_rn(lcy, half), kEps));
}

__global__ void k_edge_flags(const uint64_t* __restrict__ bits, int W, int H, int TY, uint32_t* __restrict__ flags) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)W * H) return;
    int x = (int)(i / H), y = (int)(i - (long long)x * H);
    uint32_t e = 0;
    if (occ_bit(bits, TY, x, y)) {
        for (int dx = -1; dx <= 1 && !e; ++dx)
            for (int dy = -1; dy <= 1; ++dy) {
                if (!dx && !dy) continue;
                int cx = x + dx, cy = y + dy;
                if (cx >= 0 && cy >= 0 && cx < W && cy < H && !occ_bit(bits, TY, cx, cy)) { e = 1; break; }
            }
    }
    flags[i] = e;
}

__global__ void k_compact_edges(const uint32_t* __restrict__ flags, const uint32_t* __restrict__ pos, long long n,
                                uint32_t* __restrict__ edges) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (flags[i]) edges[pos[i]] = (uint32_t)i;
}

// pass 0 counts entries per bin, pass 1 scatters them
template <int PASS>
__global__ void k_project(SliceGeom g, const uint32_t* __restrict__ edges, uint32_t nedges, int H, int nslices,
                          uint32_t* __restrict__ counts, const uint32_t* __restrict__ start,
                          float* __restrict__ zeros) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)nedges * nslices) return;
    int a = (int)(t % nslices);
    uint32_t cell = __ldg(edges + t / nslices);
    int x = (int)(cell / (uint32_t)H), y = (int)(cell - (uint32_t)x * (uint32_t)H);
    float lcx;
    int lower, upper;
    project_pixel(g, a, x, y, lcx, lower, upper);
    const int width = __ldg(g.widths + a);
    const uint32_t sb = __ldg(g.slice_base + a);
    for (int i = lower; i <= upper; ++i) {
        if (i < 0 || i >= width) continue;   // outside the slice (cannot happen for in-grid pixels)
        uint32_t b = sb + (uint32_t)i;
        if (PASS == 0) atomicAdd(counts + b, 1u);
        else zeros[__ldg(start + b) + atomicAdd(counts + b, 1u)] = lcx;
    }
}

__global__ void k_max_u32(const uint32_t* __restrict__ v, size_t n, uint32_t* out) {
    uint32_t m = 0;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        m = max(m, v[i]);
    for (int o = 16; o; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

// one block per bin: bitonic sort in shared memory, then de-duplicate in
// place; ucount[b] receives the number of distinct values
__global__ void k_sort_unique(const uint32_t* __restrict__ start, float* zeros, uint32_t* __restrict__ ucount) {
    extern __shared__ float sh[];
    const uint32_t b = blockIdx.x;
    const uint32_t lo = start[b];
    const int n = (int)(start[b + 1] - lo);
    if (n == 0) { if (threadIdx.x == 0) ucount[b] = 0; return; }
    int p = 1;
    while (p < n) p <<= 1;
    for (int i = threadIdx.x; i < p; i += blockDim.x) sh[i] = i < n ? zeros[lo + i] : __int_as_float(0x7f800000);
    __syncthreads();
    for (int k = 2; k <= p; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = threadIdx.x; i < p; i += blockDim.x) {
                int l = i ^ j;
                if (l > i) {
                    float a = sh[i], c = sh[l];
                    bool up = (i & k) == 0;
                    if (up ? (c < a) : (a < c)) { sh[i] = c; sh[l] = a; }
                }
            }
            __syncthreads();
        }
    }
    if (threadIdx.x == 0) {
        int w = 0;
        for (int i = 0; i < n; ++i) {
            if (i > 0 && sh[i] == sh[i - 1]) continue;
            zeros[lo + w++] = sh[i];
        }
        ucount[b] = (uint32_t)w;
    }
}

__global__ void k_copy_bins(const uint32_t* __restrict__ src_start, const float* __restrict__ src,
                            const uint32_t* __restrict__ dst_start, float* __restrict__ dst) {
    const uint32_t b = blockIdx.x;
    const uint32_t s = src_start[b], d = dst_start[b], n = dst_start[b + 1] - d;
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) dst[d + i] = src[s + i];
}

// ------------------------------------------------------------------ prune
// One slice per launch, one thread per cell in the reference's visiting
// order (cell = x * H + y).  A cell either skips, marks directly, or -- in
// the linear-search branch when no zero point is >= x -- reuses the index
// the last assigning cell of the slice produced (the reference leaves its
// `index` unassigned there, RangeLib.h:1242-1247, and keeps the stale value).
// tag[c] = c for cells that assign an index (val[c] = that index), -1 for
// cells that do not, and -2 for cells that need the stale index.
__global__ void k_prune_classify(SliceGeom g, int a, const uint64_t* __restrict__ bits, int W, int H, int TY,
                                 const uint32_t* __restrict__ bin_start, const float* __restrict__ zeros, float mr,
                                 uint32_t* __restrict__ used, int* __restrict__ tag, int* __restrict__ val,
                                 unsigned* __restrict__ n_need) {
    const long long ncell = (long long)W * H;
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncell) return;
    const float ca = __ldg(g.cosv + a), sa = __ldg(g.sinv + a), tr = __ldg(g.trans + a);
    int x = (int)(c / H), y = (int)(c - (long long)x * H);
    int t = -1;
    const float fx = __int2float_rn(x) + 0.5f, fy = __int2float_rn(y) + 0.5f;
    const float lx = __fsub_rn(__fmul_rn(fx, ca), __fmul_rn(fy, sa));
    const float ly = __fadd_rn(__fadd_rn(__fmul_rn(fx, sa), __fmul_rn(fy, ca)), tr);
    const unsigned li = (unsigned)__float2int_rz(ly);
    if (li < (unsigned)__ldg(g.widths + a)) {
        const uint32_t b = __ldg(g.slice_base + a) + li;
        const uint32_t base = __ldg(bin_start + b);
        const int n = (int)(__ldg(bin_start + b + 1) - base);
        const int high = n - 1;
        if (high >= 0 && !occ_bit(bits, TY, x, y)) {
            const float last = __ldg(zeros + base + high);
            if (last < lx && __fsub_rn(lx, last) < mr) {
                used[base + high] = 1;
            } else {
                int index = -1;
                if (high > kBinarySearchThreshold) {
                    int l = 0, h = n;   // lower_bound
                    while (l < h) {
                        int mid = (l + h) >> 1;
                        if (__ldg(zeros + base + mid) < lx) l = mid + 1; else h = mid;
                    }
                    index = l;
                } else {
                    for (int i = 0; i < n; ++i)
                        if (__ldg(zeros + base + i) >= lx) { index = i; break; }
                }
                if (index >= 0) {
                    if (index < n) used[base + index] = 1;
                    if (index >= 1) used[base + index - 1] = 1;
                    t = (int)c;
                    val[c] = index;
                } else {
                    t = -2;
                    atomicAdd(n_need, 1u);
                }
            }
        }
    }
    tag[c] = t;
}

// cells that need the stale index: last[c] is the last assigning cell <= c
__global__ void k_prune_stale(SliceGeom g, int a, int W, int H, const uint32_t* __restrict__ bin_start,
                              const int* __restrict__ tag, const int* __restrict__ last, const int* __restrict__ val,
                              uint32_t* __restrict__ used) {
    const long long ncell = (long long)W * H;
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncell || tag[c] != -2) return;
    const int p = last[c];
    const int index = p >= 0 ? val[p] : 0;   // the reference's index starts each slice at 0 here
    int x = (int)(c / H), y = (int)(c - (long long)x * H);
    const float ca = __ldg(g.cosv + a), sa = __ldg(g.sinv + a), tr = __ldg(g.trans + a);
    const float fx = __int2float_rn(x) + 0.5f, fy = __int2float_rn(y) + 0.5f;
    const float ly = __fadd_rn(__fadd_rn(__fmul_rn(fx, sa), __fmul_rn(fy, ca)), tr);
    const unsigned li = (unsigned)__float2int_rz(ly);
    const uint32_t b = __ldg(g.slice_base + a) + li;
    const uint32_t base = __ldg(bin_start + b);
    const int n = (int)(__ldg(bin_start + b + 1) - base);
    if (index >= 0 && index < n) used[base + index] = 1;
    if (index - 1 >= 0 && index - 1 < n) used[base + index - 1] = 1;
}

// entries of slices >= nslices are kept (they are empty after construction)
__global__ void k_keep_flags(uint32_t* __restrict__ used, uint32_t first_unpruned_entry, uint32_t n) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && i >= first_unpruned_entry) used[i] = 1;
}

__global__ void k_compact_entries(const uint32_t* __restrict__ keep, const uint32_t* __restrict__ pos, uint32_t n,
                                  const float* __restrict__ src, float* __restrict__ dst) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && keep[i]) dst[pos[i]] = src[i];
}

__global__ void k_remap_starts(const uint32_t* __restrict__ old_start, const uint32_t* __restrict__ pos,
                               uint32_t nb, uint32_t* __restrict__ new_start) {
    uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b <= nb) new_start[b] = pos[old_start[b]];
}

struct DevBuf {
    void* p = nullptr;
    ~DevBuf() { if (p) cudaFree(p); }
    cudaError_t alloc(size_t bytes) { return cudaMalloc(&p, bytes ? bytes : 4); }
    template <class T> T* as() const { return static_cast<T*>(p); }
};

#define RLC_TRY(x) do { cudaError_t _e = (x); if (_e != cudaSuccess) return _e; } while (0)

}  // namespace

template <class Op, bool INCLUSIVE>
static cudaError_t scan_impl(const typename Op::T* d_in, typename Op::T* d_out, size_t n, cudaStream_t s) {
    size_t ntiles = (n + kScanTile - 1) / kScanTile;
    if (ntiles == 0) ntiles = 1;
    DevBuf sums;
    RLC_TRY(sums.alloc((ntiles + 1) * sizeof(typename Op::T)));
    k_tile_reduce<Op><<<(unsigned)ntiles, kScanThreads, 0, s>>>(d_in, n, sums.as<typename Op::T>());
    RLC_TRY(cudaGetLastError());
    k_scan_partials<Op><<<1, kScanThreads, 0, s>>>(sums.as<typename Op::T>(), ntiles);
    RLC_TRY(cudaGetLastError());
    k_scan_tiles<Op, INCLUSIVE><<<(unsigned)ntiles, kScanThreads, 0, s>>>(d_in, n, sums.as<typename Op::T>(), d_out,
                                                                         ntiles);
    RLC_TRY(cudaGetLastError());
    return cudaStreamSynchronize(s);   // the temporary is released on return
}

cudaError_t scan_exclusive_u32(const uint32_t* d_in, uint32_t* d_out, size_t n, cudaStream_t s) {
    return scan_impl<OpSum, false>(d_in, d_out, n, s);
}

cudaError_t cddt_build(const uint64_t* d_bits, int W, int H, int TY, unsigned td, const int* d_widths,
                       const float* d_trans, const float* d_cos, const float* d_sin, const uint32_t* h_slice_base,
                       CddtBuild* out, cudaStream_t s, char* why, size_t why_len) {
    const int nslices = (int)((td + 1) / 2);   // a < td / 2.0
    const uint32_t nb = h_slice_base[td];
    const long long ncell = (long long)W * H;
    SliceGeom g{d_widths, d_trans, d_cos, d_sin, nullptr};

    DevBuf slice_base;
    RLC_TRY(slice_base.alloc((td + 1) * sizeof(uint32_t)));
    RLC_TRY(cudaMemcpyAsync(slice_base.p, h_slice_base, (td + 1) * sizeof(uint32_t), cudaMemcpyHostToDevice, s));
    g.slice_base = slice_base.as<uint32_t>();

    // 1. edge pixels, compacted in x-major order
    DevBuf flags, pos;
    RLC_TRY(flags.alloc((ncell + 1) * sizeof(uint32_t)));
    RLC_TRY(pos.alloc((ncell + 1) * sizeof(uint32_t)));
    if (ncell > 0) {
        k_edge_flags<<<blocks_for(ncell, 256), 256, 0, s>>>(d_bits, W, H, TY, flags.as<uint32_t>());
        RLC_TRY(cudaGetLastError());
    }
    RLC_TRY(scan_exclusive_u32(flags.as<uint32_t>(), pos.as<uint32_t>(), (size_t)ncell, s));
    uint32_t nedges = 0;
    RLC_TRY(cudaMemcpy(&nedges, pos.as<uint32_t>() + ncell, sizeof(uint32_t), cudaMemcpyDeviceToHost));
    DevBuf edges;
    RLC_TRY(edges.alloc((size_t)nedges * sizeof(uint32_t)));
    if (ncell > 0) {
        k_compact_edges<<<blocks_for(ncell, 256), 256, 0, s>>>(flags.as<uint32_t>(), pos.as<uint32_t>(), ncell,
                                                               edges.as<uint32_t>());
        RLC_TRY(cudaGetLastError());
    }

    // 2. count, scan, fill
    DevBuf counts, start;
    RLC_TRY(counts.alloc(((size_t)nb + 1) * sizeof(uint32_t)));
    RLC_TRY(start.alloc(((size_t)nb + 1) * sizeof(uint32_t)));
    RLC_TRY(cudaMemsetAsync(counts.p, 0, ((size_t)nb + 1) * sizeof(uint32_t), s));
    const long long work = (long long)nedges * nslices;
    if (work > 0) {
        k_project<0><<<blocks_for(work, 256), 256, 0, s>>>(g, edges.as<uint32_t>(), nedges, H, nslices,
                                                           counts.as<uint32_t>(), nullptr, nullptr);
        RLC_TRY(cudaGetLastError());
    }
    // 64-bit guard: the CSR offsets are uint32
    {
        std::vector<uint32_t> hc(nb);
        RLC_TRY(cudaMemcpy(hc.data(), counts.p, nb * sizeof(uint32_t), cudaMemcpyDeviceToHost));
        unsigned long long tot = 0;
        for (uint32_t c : hc) tot += c;
        if (tot >= 0xffffffffull) {
            snprintf(why, why_len, "CDDT table has %llu entries; the device layout holds < 2^32", tot);
            return cudaErrorInvalidValue;
        }
    }
    RLC_TRY(scan_exclusive_u32(counts.as<uint32_t>(), start.as<uint32_t>(), nb, s));
    uint32_t nraw = 0;
    RLC_TRY(cudaMemcpy(&nraw, start.as<uint32_t>() + nb, sizeof(uint32_t), cudaMemcpyDeviceToHost));
    DevBuf raw;
    RLC_TRY(raw.alloc((size_t)nraw * sizeof(float)));
    DevBuf maxlen;
    RLC_TRY(maxlen.alloc(sizeof(uint32_t)));
    RLC_TRY(cudaMemsetAsync(maxlen.p, 0, sizeof(uint32_t), s));
    if (nb > 0) {
        k_max_u32<<<256, 256, 0, s>>>(counts.as<uint32_t>(), nb, maxlen.as<uint32_t>());
        RLC_TRY(cudaGetLastError());
    }
    RLC_TRY(cudaMemsetAsync(counts.p, 0, ((size_t)nb + 1) * sizeof(uint32_t), s));
    if (work > 0) {
        k_project<1><<<blocks_for(work, 256), 256, 0, s>>>(g, edges.as<uint32_t>(), nedges, H, nslices,
                                                           counts.as<uint32_t>(), start.as<uint32_t>(),
                                                           raw.as<float>());
        RLC_TRY(cudaGetLastError());
    }

    // 3. sort + unique per bin
    uint32_t mlen = 0;
    RLC_TRY(cudaMemcpy(&mlen, maxlen.p, sizeof(uint32_t), cudaMemcpyDeviceToHost));
    size_t p2 = 1;
    while (p2 < mlen) p2 <<= 1;
    size_t smem = p2 * sizeof(float);
    if (smem > 200 * 1024) {
        snprintf(why, why_len, "CDDT bin of %u zero points exceeds the in-shared-memory sort (max 51200)", mlen);
        return cudaErrorInvalidValue;
    }
    DevBuf ucount;
    RLC_TRY(ucount.alloc(((size_t)nb + 1) * sizeof(uint32_t)));
    if (nb > 0) {
        if (smem > 48 * 1024)
            RLC_TRY(cudaFuncSetAttribute(k_sort_unique, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k_sort_unique<<<nb, 128, smem, s>>>(start.as<uint32_t>(), raw.as<float>(), ucount.as<uint32_t>());
        RLC_TRY(cudaGetLastError());
    }

    // 4. final CSR
    uint32_t* d_bin_start = nullptr;
    float* d_zeros = nullptr;
    RLC_TRY(cudaMalloc(&d_bin_start, ((size_t)nb + 1) * sizeof(uint32_t)));
    cudaError_t e = scan_exclusive_u32(ucount.as<uint32_t>(), d_bin_start, nb, s);
    uint32_t nz = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&nz, d_bin_start + nb, sizeof(uint32_t), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMalloc(&d_zeros, cddt_zeros_bytes(nz));
    if (e == cudaSuccess && nb > 0) {
        k_copy_bins<<<nb, 128, 0, s>>>(start.as<uint32_t>(), raw.as<float>(), d_bin_start, d_zeros);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    uint32_t* d_slice_base = nullptr;
    if (e == cudaSuccess) e = cudaMalloc(&d_slice_base, (td + 1) * sizeof(uint32_t));
    if (e == cudaSuccess)
        e = cudaMemcpy(d_slice_base, h_slice_base, (td + 1) * sizeof(uint32_t), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaFree(d_bin_start);
        cudaFree(d_zeros);
        cudaFree(d_slice_base);
        return e;
    }
    out->slice_base = d_slice_base;
    out->bin_start = d_bin_start;
    out->zeros = d_zeros;
    out->total_bins = nb;
    out->nzeros = nz;
    return cudaSuccess;
}

cudaError_t cddt_prune(const uint64_t* d_bits, int W, int H, int TY, unsigned td, float max_range,
                       const int* d_widths, const float* d_trans, const float* d_cos, const float* d_sin,
                       CddtBuild* tab, cudaStream_t s) {
    const int nslices = (int)((td + 1) / 2);
    const uint32_t nz = tab->nzeros, nb = tab->total_bins;
    SliceGeom g{d_widths, d_trans, d_cos, d_sin, tab->slice_base};
    DevBuf used, pos;
    RLC_TRY(used.alloc(((size_t)nz + 1) * sizeof(uint32_t)));
    RLC_TRY(pos.alloc(((size_t)nz + 1) * sizeof(uint32_t)));
    RLC_TRY(cudaMemsetAsync(used.p, 0, ((size_t)nz + 1) * sizeof(uint32_t), s));
    const long long ncell = (long long)W * H;
    if (ncell > 0 && nz > 0) {
        DevBuf tag, val, last, need;
        RLC_TRY(tag.alloc((size_t)ncell * sizeof(int)));
        RLC_TRY(val.alloc((size_t)ncell * sizeof(int)));
        RLC_TRY(last.alloc((size_t)ncell * sizeof(int)));
        RLC_TRY(need.alloc(sizeof(unsigned)));
        for (int a = 0; a < nslices; ++a) {
            RLC_TRY(cudaMemsetAsync(need.p, 0, sizeof(unsigned), s));
            k_prune_classify<<<blocks_for(ncell, 256), 256, 0, s>>>(g, a, d_bits, W, H, TY, tab->bin_start,
                                                                    tab->zeros, max_range, used.as<uint32_t>(),
                                                                    tag.as<int>(), val.as<int>(), need.as<unsigned>());
            RLC_TRY(cudaGetLastError());
            unsigned n_need = 0;
            RLC_TRY(cudaMemcpyAsync(&n_need, need.p, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
            RLC_TRY(cudaStreamSynchronize(s));
            if (n_need == 0) continue;
            RLC_TRY((scan_impl<OpMax, true>(tag.as<int>(), last.as<int>(), (size_t)ncell, s)));
            k_prune_stale<<<blocks_for(ncell, 256), 256, 0, s>>>(g, a, W, H, tab->bin_start, tag.as<int>(),
                                                                 last.as<int>(), val.as<int>(), used.as<uint32_t>());
            RLC_TRY(cudaGetLastError());
        }
    }
    // slices >= nslices keep all their entries
    uint32_t first_unpruned = 0;
    {
        uint32_t first_bin = 0;
        std::vector<uint32_t> hsb(td + 1);
        RLC_TRY(cudaMemcpy(hsb.data(), tab->slice_base, (td + 1) * sizeof(uint32_t), cudaMemcpyDeviceToHost));
        first_bin = hsb[nslices];
        RLC_TRY(cudaMemcpy(&first_unpruned, tab->bin_start + first_bin, sizeof(uint32_t), cudaMemcpyDeviceToHost));
    }
    if (nz > 0) {
        k_keep_flags<<<blocks_for(nz, 256), 256, 0, s>>>(used.as<uint32_t>(), first_unpruned, nz);
        RLC_TRY(cudaGetLastError());
    }
    RLC_TRY(scan_exclusive_u32(used.as<uint32_t>(), pos.as<uint32_t>(), nz, s));
    uint32_t nkeep = 0;
    RLC_TRY(cudaMemcpy(&nkeep, pos.as<uint32_t>() + nz, sizeof(uint32_t), cudaMemcpyDeviceToHost));
    float* d_new = nullptr;
    uint32_t* d_new_start = nullptr;
    RLC_TRY(cudaMalloc(&d_new, cddt_zeros_bytes(nkeep)));
    cudaError_t e = cudaMalloc(&d_new_start, ((size_t)nb + 1) * sizeof(uint32_t));
    if (e == cudaSuccess && nz > 0) {
        k_compact_entries<<<blocks_for(nz, 256), 256, 0, s>>>(used.as<uint32_t>(), pos.as<uint32_t>(), nz,
                                                              tab->zeros, d_new);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
        k_remap_starts<<<blocks_for((long long)nb + 1, 256), 256, 0, s>>>(tab->bin_start, pos.as<uint32_t>(), nb,
                                                                           d_new_start);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        cudaFree(d_new);
        cudaFree(d_new_start);
        return e;
    }
    cudaFree(tab->zeros);
    cudaFree(tab->bin_start);
    tab->zeros = d_new;
    tab->bin_start = d_new_start;
    tab->nzeros = nkeep;
    return cudaSuccess;
}

}  // namespace rlc
