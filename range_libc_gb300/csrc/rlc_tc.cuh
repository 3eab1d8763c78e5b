// tcgen05 (5th-generation tensor core) building blocks for sm_103a, written
// as inline PTX: shared-memory matrix descriptors, the kind::f16 instruction
// descriptor, TMEM allocation, MMA issue/commit, mbarrier waits with a time
// bound, TMEM loads, and TMA tile loads.
//
// Shared-memory operand layout used throughout (no swizzle, K-major): a tile
// of R rows x 64 K (bf16) is stored as 8x8 "core matrices" of 128 contiguous
// bytes (8 rows x 16 B); core matrix (i, j) -- rows 8i..8i+7, k 8j..8j+7 --
// sits at byte (i * 8 + j) * 128.  Adjacent core matrices along K are 128 B
// apart (leading byte offset), along M/N 1024 B apart (stride byte offset).
#pragma once

#include <cuda_bf16.h>
#include <stdint.h>

namespace rlc {
namespace tc {

constexpr int kKChunk = 64;                   // K elements per smem stage
constexpr uint32_t kCoreBytes = 128;          // one 8x8 bf16 core matrix
constexpr uint32_t kRowBlockBytes = 8 * kCoreBytes;   // 8 core matrices along K

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

// byte offset of element (row, k) of a K-major core-matrix tile (k < 64)
__device__ __forceinline__ uint32_t core_offset(int row, int k) {
    return (uint32_t)(((row >> 3) * 8 + (k >> 3)) * kCoreBytes + (row & 7) * 16 + (k & 7) * 2);
}

// Shared-memory matrix descriptor: start address, leading / stride byte
// offsets (all >> 4), descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t make_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFF);
    d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
    d |= (uint64_t)1 << 46;   // version
    return d;                 // base offset 0, layout type 0 (no swizzle)
}

// Descriptor of a K-major operand in the 128-byte swizzled layout that a TMA load with
// CU_TENSOR_MAP_SWIZZLE_128B and a 64-element (128-byte) inner box writes: row r of the tile at
// r * 128 bytes, its eight 16-byte chunks permuted by (chunk ^ (r & 7)); 8-row groups 1024 bytes
// apart (SBO); the tile 1024-byte aligned.  Successive 16-element K steps start 32 bytes further
// into the row (the hardware applies the swizzle to the resulting addresses).
__device__ __forceinline__ uint64_t make_desc_sw128(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFF);
    d |= (uint64_t)1 << 16;                        // leading byte offset (unused by swizzled K-major)
    d |= (uint64_t)(1024 >> 4) << 32;              // stride byte offset: 8 rows x 128 bytes
    d |= (uint64_t)1 << 46;                        // version
    d |= (uint64_t)2 << 61;                        // 128-byte swizzle
    return d;
}

// kind::f16 instruction descriptor: D f32, A and B bf16, both K-major, M x N
__host__ __device__ constexpr uint32_t make_idesc(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
        "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate));
}

// arrive on the mbarrier once every previously issued MMA of this thread completes
__device__ __forceinline__ void mma_commit(uint32_t mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
                 : "memory");
}

__device__ __forceinline__ void mbar_init(uint32_t mbar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mbar), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Wait for phase `parity` of the mbarrier, giving up after ~2^31 clock
// cycles (about one second): returns false on time-out.
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity) {
    const long long t0 = clock64();
    for (;;) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(mbar), "r"(parity)
            : "memory");
        if (done) return true;
        if (clock64() - t0 > (1ll << 31)) return false;
    }
}

// make generic-proxy shared-memory writes visible to the tensor core (async proxy)
__device__ __forceinline__ void fence_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void fence_before_sync() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void fence_after_sync() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// TMEM allocation by one full warp; the address lands in *dst (shared memory)
__device__ __forceinline__ void tmem_alloc(uint32_t dst_smem, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(dst_smem), "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// 32 lanes x 32 consecutive 32-bit columns: thread l of the warp gets row
// (lane base + l), columns [col, col + 32)
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// ---- TMA (cp.async.bulk.tensor) ---------------------------------------------
// arrive on the mbarrier (count 1) and expect `bytes` of asynchronous copies to complete on it
__device__ __forceinline__ void mbar_arrive_expect_tx(uint32_t mbar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar), "r"(bytes) : "memory");
}

// 2-D tiled TMA load of the box at (x = innermost coordinate, y) of the tensor map into shared
// memory at dst, completing `bytes` of transaction count on the mbarrier.  x times the element
// size must be a multiple of 16 bytes; dst 128-byte aligned.
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const void* tmap, int x, int y, uint32_t mbar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
        ::"r"(dst), "l"(reinterpret_cast<uint64_t>(tmap)), "r"(x), "r"(y), "r"(mbar)
        : "memory");
}

__device__ __forceinline__ void tma_prefetch_map(const void* tmap) {
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(tmap)) : "memory");
}

}  // namespace tc
}  // namespace rlc
