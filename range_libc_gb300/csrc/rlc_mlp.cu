// Learned range surrogate: a per-map MLP that predicts where a ray meets a
// wall, trained on rays cast by the exact GPU ray marcher, with hand-written
// tcgen05 (TMEM-accumulating) BF16 GEMMs for the forward and backward passes
// and an Adam kernel.  No counterpart in the reference.
//
// Model: the grid-frame ray (x, y, theta) becomes u = (x/W, y/H, cos, sin);
// each of the 4 inputs is expanded by 64 sinusoidal frequencies f_k =
// fmax^(k/63) (sin and cos of pi f_k u) into 512 features, then four hidden
// layers of width 256 with GELU (tanh form), then one linear output: the
// march parameter t at which the exact marcher reaches its hit cell (pixels).
// Weights and activations are BF16, accumulation and the output layer FP32.
//
// A prediction t^ is accepted when the cell at x0 + t^ dir is occupied and
// the cell at x0 + (t^ - 1) dir is free; the range returned is then the
// reference's distance to that cell's corner, otherwise the ray is recast
// exactly (compacted into a dense second pass).
#include "rangelibc.h"
#include "rlc_internal.cuh"
#include "rlc_tc.cuh"

#include <cuda.h>
#include <cuda_bf16.h>

#include <atomic>
#include <cmath>
#include <mutex>
#include <cstdio>
#include <cstring>
#include <vector>

namespace rlc {
namespace {

typedef __nv_bfloat16 bf16;

constexpr int kFeat = 512;      // 4 inputs x 64 frequencies x {sin, cos}
constexpr int kHidden = 256;
constexpr int kLayers = 4;      // hidden layers
constexpr int kBM = 128;        // GEMM tile rows (TMEM lanes)
constexpr int kBN = 256;        // GEMM tile columns (TMEM columns)

// flat fp32 parameter layout
constexpr size_t kW0 = (size_t)kHidden * kFeat;              // layer 0: 256 x 512 (out x in)
constexpr size_t kWh = (size_t)kHidden * kHidden;            // layers 1-3: 256 x 256
constexpr size_t kParamCount = kW0 + kHidden + 3 * (kWh + kHidden) + kHidden + 1;

__host__ __device__ inline size_t w_offset(int l) { return l == 0 ? 0 : kW0 + kHidden + (size_t)(l - 1) * (kWh + kHidden); }
__host__ __device__ inline size_t b_offset(int l) { return w_offset(l) + (l == 0 ? kW0 : kWh); }
__host__ __device__ inline int layer_in(int l) { return l == 0 ? kFeat : kHidden; }
constexpr size_t kOutW = kW0 + kHidden + 3 * (kWh + kHidden);  // output weights [256], then bias [1]

// -------------------------------------------------------------------- GEMM
enum Epi : int { EPI_F32 = 0, EPI_FWD = 1, EPI_BWD = 2, EPI_F32_ADD = 3 };

struct GemmArgs {
    const bf16* A;   // A[m * lda + k] (a_t and b_t must be 0: both operands K-major)
    const bf16* B;   // B[n * ldb + k]
    int lda, ldb, a_t, b_t;
    int M, N, K;
    int ksplit;         // K range of blockIdx.z: [z * ksplit, (z + 1) * ksplit)
    int epi;
    int ldc;
    float* C32;         // EPI_F32: C[m * ldc + n]; EPI_F32_ADD: C[m * ldc + n] += (split-K partials)
    const float* bias;  // EPI_FWD
    bf16* Zout;         // EPI_FWD: pre-activation
    bf16* Hout;         // EPI_FWD: GELU(z)
    const bf16* Zin;    // EPI_BWD: pre-activation of the layer below
    bf16* dZ;           // EPI_BWD: acc * GELU'(Zin)
    bf16* HoutT;        // EPI_FWD (optional): GELU(z) transposed, [n * ldt + m]
    bf16* dZT;          // EPI_BWD (optional): dZ transposed, [n * ldt + m]
    int ldt;
    unsigned* err;
};

// GELU (tanh form).  tanh is the SFU's single-instruction approximation
// (PTX tanh.approx.f32, relative error about 2^-11, below the BF16 rounding
// of the activations); training and inference use the same function.
__device__ __forceinline__ float tanh_sfu(float x) {
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

__device__ __forceinline__ float gelu(float z) {
    const float k0 = 0.7978845608028654f, k1 = 0.044715f;
    return 0.5f * z * (1.0f + tanh_sfu(k0 * (z + k1 * z * z * z)));
}

__device__ __forceinline__ float gelu_grad(float z) {
    const float k0 = 0.7978845608028654f, k1 = 0.044715f;
    float u = k0 * (z + k1 * z * z * z);
    float th = tanh_sfu(u);
    return 0.5f * (1.0f + th) + 0.5f * z * (1.0f - th * th) * k0 * (1.0f + 3.0f * k1 * z * z);
}

// --------------------------------------------------------------- TMA GEMM
// C tile [128 x 256] at (blockIdx.y * 128, blockIdx.x * 256) of C = A . B^T, both operands
// K-major in global memory (A[m * lda + k], B[n * ldb + k]), K range [z * ksplit, (z+1) * ksplit).
//
// Warp-specialised (192 threads, pipeline stages of 48 KB):
//   warp 0     TMA producer: per 64-wide K chunk, one tile load of A (128 rows x 128 bytes) and
//              one of B (256 rows) into stage s, completing on full[s]; it reuses a stage once the
//              MMAs that read it have committed to empty[s];
//   warp 1     allocates 256 TMEM columns; one thread issues the chunk's four
//              tcgen05.mma (K = 16 each) per stage and commits them to empty[s], and after the
//              last chunk to `accum`;
//   warps 2-5  epilogue: wait for `accum`, read the accumulator with tcgen05.ld (warp w reads
//              TMEM lanes 32 (w % 4) .. + 31) and apply the epilogue.
// Shared-memory operand layout (K-major, 128-byte swizzle, as the TMA writes it): row r of a
// stage's tile at r * 128 bytes with its 16-byte chunks permuted by r & 7 (tc::make_desc_sw128).
// Every wait is bounded (about a second); a time-out sets bit 16 of *err, the remaining roles stop
// at their next wait, and the CTA still frees its TMEM.
//
// kStages = 4 (one CTA per SM) for the long-K weight gradients; 2 (two CTAs per SM, so that one
// CTA's epilogue overlaps the other's loads and MMAs) for the short-K forward and input-gradient
// GEMMs (K = 256 or 512).
constexpr uint32_t kStageA = kBM * tc::kKChunk * 2;   // 16 KB
constexpr uint32_t kStageB = kBN * tc::kKChunk * 2;   // 32 KB
template <int kStages>
constexpr size_t tma_smem() { return kStages * (size_t)(kStageA + kStageB) + 1024; }   // + alignment slack
constexpr int kGemmThreads = 192;

template <int kStages>
__global__ void __launch_bounds__(kGemmThreads, kStages <= 2 ? 2 : 1)
k_gemm_tma(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, GemmArgs g) {
    extern __shared__ uint8_t smem_raw[];
    __shared__ __align__(8) uint64_t full[kStages], empty[kStages], accum;
    __shared__ uint32_t tmem_base;
    __shared__ int abort_flag, n_issued, n_consumed;
    uint8_t* smem = reinterpret_cast<uint8_t*>(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    const uint32_t sbase = tc::smem_addr(smem);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m0 = blockIdx.y * kBM, n0 = blockIdx.x * kBN;
    const int kbase = blockIdx.z * g.ksplit;
    const int nchunks = g.ksplit / tc::kKChunk;
    if (warp == 1) tc::tmem_alloc(tc::smem_addr(&tmem_base), 256);
    if (threadIdx.x == 0) {
        for (int i = 0; i < kStages; ++i) {
            tc::mbar_init(tc::smem_addr(&full[i]), 1);
            tc::mbar_init(tc::smem_addr(&empty[i]), 1);
        }
        tc::mbar_init(tc::smem_addr(&accum), 1);
        abort_flag = 0;
        n_issued = 0;
        n_consumed = 0;
        tc::fence_mbar_init();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = tmem_base;
    auto stage_a = [&](int st) { return sbase + (uint32_t)st * (kStageA + kStageB); };
    auto stage_b = [&](int st) { return stage_a(st) + kStageA; };
    if (warp == 0 && lane == 0) {
        // ---- producer
        tc::tma_prefetch_map(&tmA);
        tc::tma_prefetch_map(&tmB);
        for (int c = 0; c < nchunks; ++c) {
            const int st = c % kStages;
            if (c >= kStages && !tc::mbar_wait(tc::smem_addr(&empty[st]), ((c / kStages) - 1) & 1)) {
                atomicOr(g.err, 16u);
                atomicExch(&abort_flag, 1);
                break;
            }
            if (*(volatile int*)&abort_flag) break;
            const uint32_t fb = tc::smem_addr(&full[st]);
            tc::mbar_arrive_expect_tx(fb, kStageA + kStageB);
            const int k0 = kbase + c * tc::kKChunk;
            tc::tma_load_2d(stage_a(st), &tmA, k0, m0, fb);
            tc::tma_load_2d(stage_b(st), &tmB, k0, n0, fb);
            n_issued = c + 1;
        }
    } else if (warp == 1 && lane == 0) {
        // ---- MMA issuer
        const uint32_t idesc = tc::make_idesc(kBM, kBN);
        for (int c = 0; c < nchunks; ++c) {
            const int st = c % kStages;
            if (!tc::mbar_wait(tc::smem_addr(&full[st]), (c / kStages) & 1)) {
                atomicOr(g.err, 16u);
                atomicExch(&abort_flag, 1);
                break;
            }
            tc::fence_after_sync();
#pragma unroll
            for (int ks = 0; ks < tc::kKChunk / 16; ++ks) {
                const uint64_t ad = tc::make_desc_sw128(stage_a(st) + ks * 32);
                const uint64_t bd = tc::make_desc_sw128(stage_b(st) + ks * 32);
                tc::mma_bf16(tmem, ad, bd, idesc, (c > 0 || ks > 0) ? 1u : 0u);
            }
            tc::mma_commit(tc::smem_addr(&empty[st]));
            n_consumed = c + 1;
        }
        // `accum` completes once every MMA issued above has (also with none issued)
        tc::mma_commit(tc::smem_addr(&accum));
    } else if (warp >= 2) {
        // ---- epilogue
        const bool ok = tc::mbar_wait(tc::smem_addr(&accum), 0);
        tc::fence_after_sync();
        if (!ok) {
            if (lane == 0) atomicOr(g.err, 16u);
        } else if (!*(volatile int*)&abort_flag && nchunks > 0) {
            const int lq = warp & 3;   // TMEM lane quarter this warp may read
            const int row = m0 + lq * 32 + lane;
            const uint32_t lane_addr = tmem + ((uint32_t)(lq * 32) << 16);
            for (int cb = 0; cb < kBN; cb += 32) {
                float v[32];
                tc::tmem_ld32(lane_addr + cb, v);
                const int col0 = n0 + cb;
                if (g.epi == EPI_F32) {
                    float* out = g.C32 + (size_t)row * g.ldc + col0;
#pragma unroll
                    for (int i = 0; i < 32; i += 4) *reinterpret_cast<float4*>(out + i) = make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]);
                } else if (g.epi == EPI_F32_ADD) {   // split-K partial sums: 16-byte vector reductions
                    float* out = g.C32 + (size_t)row * g.ldc + col0;
#pragma unroll
                    for (int i = 0; i < 32; i += 4)
                        asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(out + i), "f"(v[i]),
                                     "f"(v[i + 1]), "f"(v[i + 2]), "f"(v[i + 3])
                                     : "memory");
                } else if (g.epi == EPI_FWD) {
                    __nv_bfloat162 zp[16], hp[16];
#pragma unroll
                    for (int i = 0; i < 32; i += 2) {
                        const float z0 = v[i] + __ldg(g.bias + col0 + i), z1 = v[i + 1] + __ldg(g.bias + col0 + i + 1);
                        zp[i / 2] = __floats2bfloat162_rn(z0, z1);
                        const float2 zf = __bfloat1622float2(zp[i / 2]);   // GELU of the stored (rounded) pre-activation
                        hp[i / 2] = __floats2bfloat162_rn(gelu(zf.x), gelu(zf.y));
                        if (g.HoutT) {   // transposed copy [column][row] for the weight-gradient GEMMs
                            g.HoutT[(size_t)(col0 + i) * g.ldt + row] = __low2bfloat16(hp[i / 2]);
                            g.HoutT[(size_t)(col0 + i + 1) * g.ldt + row] = __high2bfloat16(hp[i / 2]);
                        }
                    }
                    uint4* zo = reinterpret_cast<uint4*>(g.Zout + (size_t)row * g.ldc + col0);
                    uint4* ho = reinterpret_cast<uint4*>(g.Hout + (size_t)row * g.ldc + col0);
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        zo[q] = *reinterpret_cast<const uint4*>(zp + 4 * q);
                        ho[q] = *reinterpret_cast<const uint4*>(hp + 4 * q);
                    }
                } else {
                    const uint4* zi = reinterpret_cast<const uint4*>(g.Zin + (size_t)row * g.ldc + col0);
                    __nv_bfloat162 zin[16], dp[16];
#pragma unroll
                    for (int q = 0; q < 4; ++q) *reinterpret_cast<uint4*>(zin + 4 * q) = zi[q];
#pragma unroll
                    for (int i = 0; i < 32; i += 2) {
                        const float2 z = __bfloat1622float2(zin[i / 2]);
                        dp[i / 2] = __floats2bfloat162_rn(v[i] * gelu_grad(z.x), v[i + 1] * gelu_grad(z.y));
                        if (g.dZT) {
                            g.dZT[(size_t)(col0 + i) * g.ldt + row] = __low2bfloat16(dp[i / 2]);
                            g.dZT[(size_t)(col0 + i + 1) * g.ldt + row] = __high2bfloat16(dp[i / 2]);
                        }
                    }
                    uint4* dz = reinterpret_cast<uint4*>(g.dZ + (size_t)row * g.ldc + col0);
#pragma unroll
                    for (int q = 0; q < 4; ++q) dz[q] = *reinterpret_cast<const uint4*>(dp + 4 * q);
                }
            }
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (abort_flag && threadIdx.x == 0) {
        // tile loads issued but never waited for are still landing in this CTA's shared memory:
        // wait for them (bounded) before the CTA exits
        for (int c = n_consumed; c < n_issued; ++c) (void)tc::mbar_wait(tc::smem_addr(&full[c % kStages]), (c / kStages) & 1);
    }
    __syncthreads();
    if (warp == 1) tc::tmem_dealloc(tmem, 256);
}

// [rows x cols] -> [cols x rows] (bf16), 32 x 32 tiles through shared memory
__global__ void k_transpose_bf16(const bf16* __restrict__ src, int rows, int cols, int lds, bf16* __restrict__ dst,
                                 int ldd) {
    __shared__ bf16 t[32][33];
    const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
        const int r = r0 + i, c = c0 + threadIdx.x;
        if (r < rows && c < cols) t[i][threadIdx.x] = src[(size_t)r * lds + c];
    }
    __syncthreads();
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
        const int c = c0 + i, r = r0 + threadIdx.x;
        if (r < rows && c < cols) dst[(size_t)c * ldd + r] = t[threadIdx.x][i];
    }
}

cudaError_t transpose_bf16(const bf16* src, int rows, int cols, int lds, bf16* dst, int ldd, cudaStream_t s) {
    if (rows <= 0 || cols <= 0) return cudaSuccess;
    k_transpose_bf16<<<dim3((cols + 31) / 32, (rows + 31) / 32), dim3(32, 8), 0, s>>>(src, rows, cols, lds, dst, ldd);
    return cudaGetLastError();
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link to the driver library)
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_tiled() {
    static EncodeTiledFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess && q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
        else
            cudaGetLastError();
    });
    return fn;
}

// tensor map of a K-major bf16 operand [rows x K] (row stride ld elements): boxes of 64 K x
// box_rows, 128-byte swizzled in shared memory
cudaError_t operand_map(CUtensorMap* map, const bf16* base, int rows, int K, int ld, int box_rows) {
    EncodeTiledFn enc = encode_tiled();
    if (!enc) return cudaErrorNotSupported;
    if (((uintptr_t)base & 15) || (ld * 2) % 16) return cudaErrorInvalidValue;
    const cuuint64_t dim[2] = {(cuuint64_t)K, (cuuint64_t)rows};
    const cuuint64_t stride[1] = {(cuuint64_t)ld * 2};
    const cuuint32_t box[2] = {(cuuint32_t)tc::kKChunk, (cuuint32_t)box_rows};   // 128-byte rows
    const cuuint32_t estr[2] = {1, 1};
    const CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<bf16*>(base), dim, stride, box, estr,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

cudaError_t gemm(GemmArgs g, cudaStream_t s) {
    if (g.M % kBM || g.N % kBN || g.K % tc::kKChunk || g.K <= 0) return cudaErrorInvalidValue;
    if (g.a_t || g.b_t) return cudaErrorInvalidValue;   // operands are K-major (transposed copies are made)
    if (g.ksplit <= 0) g.ksplit = g.K;
    if (g.K % g.ksplit || g.ksplit % tc::kKChunk) return cudaErrorInvalidValue;
    if (g.ksplit != g.K && g.epi != EPI_F32_ADD) return cudaErrorInvalidValue;
    CUtensorMap ta, tb;
    if (cudaError_t e = operand_map(&ta, g.A, g.M, g.K, g.lda, kBM)) return e;
    if (cudaError_t e = operand_map(&tb, g.B, g.N, g.K, g.ldb, kBN)) return e;
    static std::atomic<unsigned long long> attr2{0}, attr4{0};
    dim3 grid(g.N / kBN, g.M / kBM, g.K / g.ksplit);
    if (g.ksplit / tc::kKChunk > 8) {
        if (cudaError_t e = ensure_smem_attr(k_gemm_tma<4>, (int)tma_smem<4>(), attr4)) return e;
        k_gemm_tma<4><<<grid, kGemmThreads, tma_smem<4>(), s>>>(ta, tb, g);
    } else {
        if (cudaError_t e = ensure_smem_attr(k_gemm_tma<2>, (int)tma_smem<2>(), attr2)) return e;
        k_gemm_tma<2><<<grid, kGemmThreads, tma_smem<2>(), s>>>(ta, tb, g);
    }
    return cudaGetLastError();
}

// ---------------------------------------------------------------- features
struct FeatParams {
    float inv_w, inv_h;
    float freq[64];
};

__device__ __forceinline__ void ray_features(const FeatParams& fp, float x, float y, float th, bf16* out) {
    float s, c;
    sincosf(th, &s, &c);
    const float u[4] = {x * fp.inv_w, y * fp.inv_h, c, s};
#pragma unroll
    for (int d = 0; d < 4; ++d) {
        for (int k = 0; k < 64; k += 2) {
            float s0, c0, s1, c1;
            sincospif(fp.freq[k] * u[d], &s0, &c0);
            sincospif(fp.freq[k + 1] * u[d], &s1, &c1);
            __nv_bfloat162* o = reinterpret_cast<__nv_bfloat162*>(out + d * 128 + k * 2);
            o[0] = __floats2bfloat162_rn(s0, c0);
            o[1] = __floats2bfloat162_rn(s1, c1);
        }
    }
}

// rays given as grid-frame (x, y, theta) triples
__global__ void k_features(FeatParams fp, const float* __restrict__ xyt, int n, int n_pad, bf16* __restrict__ X) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n_pad) return;
    bf16* out = X + (size_t)r * kFeat;
    if (r >= n) {
        for (int j = 0; j < kFeat; j += 8) *reinterpret_cast<uint4*>(out + j) = make_uint4(0, 0, 0, 0);
        return;
    }
    ray_features(fp, xyt[3 * (size_t)r], xyt[3 * (size_t)r + 1], xyt[3 * (size_t)r + 2], out);
}

// ------------------------------------------------------ fused forward pass
// Inference of the whole network for 128 rays per CTA without leaving the SM:
// the features of one 32-wide K stage are computed straight into the A
// operand (shared memory, core-matrix layout), each layer accumulates its
// 128 x 256 output in TMEM, and the epilogue (bias, BF16 rounding, GELU)
// writes the next layer's A operand back into shared memory; the output
// layer is a per-row dot product in the last epilogue.  Only the rays' poses
// come in and one float per ray goes out (the layer-by-layer path moves
// ~3.1 KB per ray through HBM).  Weights stream from L2 with cp.async into two
// 16 KB stages of 256 x 32: stage c+1 is copied while the MMAs of stage c run.
// Two threads share each TMEM lane (row) and split its features and epilogue
// columns.  Every MMA operand, rounding point and summation order matches the
// layer-by-layer path, so the predictions are bit-identical to it.
// 96 KB of shared memory and 256 TMEM columns per CTA: two CTAs per SM, so
// one CTA's epilogue or operand loads overlap the other's MMAs.
constexpr int kFwdThreads = 256;   // two threads per TMEM lane (row): column halves
constexpr int kFK = 32;            // K elements per pipeline stage
constexpr uint32_t kFStage = 512;  // bytes between 8-row groups of a 32-wide K tile (4 core matrices)
constexpr size_t kFwdSmem = 2 * 16384 + 65536;   // two 256 x 32 weight stages + activations

// byte offset of element (row, k) (k < 32) in a 32-wide K tile of core matrices
__device__ __forceinline__ uint32_t core32(int row, int k) {
    return (uint32_t)((row >> 3) * kFStage + (k >> 3) * tc::kCoreBytes + (row & 7) * 16 + (k & 7) * 2);
}

// bf16 element k (< 256) of row `row` of the activation buffer (4 K chunks of 64 in core layout)
__device__ __forceinline__ uint32_t act_offset(int row, int k) {
    return (uint32_t)(k >> 6) * 16384u + tc::core_offset(row, k & 63);
}

// 16 features [32c + 16h, 32c + 16h + 16) of a ray with inputs u: input d = c / 4,
// frequencies (c % 4) * 16 + 8h .. + 8, as 2 rows of 16 bytes of the core layout
__device__ __forceinline__ void feature_quarter(const FeatParams& fp, const float* u, int c, int h, uint4* out) {
    const int d = c >> 2, k0 = (c & 3) * 16 + 8 * h;
#pragma unroll
    for (int v = 0; v < 2; ++v) {
        __nv_bfloat162 hb[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            float sn, cs;
            sincospif(fp.freq[k0 + 4 * v + q] * u[d], &sn, &cs);
            hb[q] = __floats2bfloat162_rn(sn, cs);
        }
        out[v] = *reinterpret_cast<const uint4*>(hb);
    }
}

__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// weight rows [0, 256) x K [k0, k0 + 32) of a layer (row-major [256][ld]) into a stage, asynchronously
__device__ __forceinline__ void load_weights32(uint32_t dst, const bf16* __restrict__ w, int ld, int k0) {
    for (int v = threadIdx.x; v < kBN * (kFK / 8); v += blockDim.x) {
        const int row = v >> 2, kv = v & 3;
        cp_async16(dst + (uint32_t)((row >> 3) * kFStage + kv * tc::kCoreBytes + (row & 7) * 16),
                   w + (size_t)row * ld + k0 + kv * 8);
    }
}

// One layer's MMA chunks, pipelined: the weights of chunk c + 1 are copied into
// the other stage while the MMAs of chunk c run; a stage is refilled only after
// the MMAs that read it have completed (one mbarrier per stage).  Layer 0
// computes its A operand (features) per chunk into sA[c % 2] inside the
// activation buffer; hidden layers read A from the activations.
struct FwdPipe {
    uint32_t sB[2], mbar[2], par[2];
    uint32_t tmem, idesc;
};

template <bool FEATURES>
__device__ __forceinline__ bool fwd_layer(FwdPipe& P, const bf16* __restrict__ w, int K, uint32_t sH, uint8_t* sA_gen,
                                          const FeatParams& fp, const float* u, bool live, int row, int half) {
    const int C = K / kFK;
    bool ok = true;
    load_weights32(P.sB[0], w, K, 0);
    cp_async_commit();
    for (int c = 0; c < C; ++c) {
        const int st = c & 1;
        if (c + 1 < C) {
            if (c >= 1) {   // stage st ^ 1 was read by the MMAs of chunk c - 1
                const bool wt = tc::mbar_wait(P.mbar[st ^ 1], P.par[st ^ 1]);
                P.par[st ^ 1] ^= 1u;
                if (!__syncthreads_and(wt)) return false;
            }
            load_weights32(P.sB[st ^ 1], w, K, (c + 1) * kFK);
            cp_async_commit();
        }
        uint32_t a0;
        if (FEATURES) {   // A stage st (inside the activation buffer) was read by chunk c - 2, complete by now
            uint4 f[2];
            if (live) {
                feature_quarter(fp, u, c, half, f);
            } else {
                f[0] = f[1] = make_uint4(0, 0, 0, 0);
            }
            uint8_t* sa = sA_gen + st * 8192;
            *reinterpret_cast<uint4*>(sa + core32(row, 16 * half)) = f[0];
            *reinterpret_cast<uint4*>(sa + core32(row, 16 * half + 8)) = f[1];
            a0 = tc::smem_addr(sa);
        } else {
            a0 = sH + (uint32_t)(c >> 1) * 16384u + (uint32_t)(c & 1) * 4u * tc::kCoreBytes;
        }
        if (c + 1 < C) cp_async_wait<1>(); else cp_async_wait<0>();
        tc::fence_async_smem();
        __syncthreads();
        if (threadIdx.x == 0) {
            tc::fence_after_sync();
            const uint32_t sbo_a = FEATURES ? kFStage : tc::kRowBlockBytes;
#pragma unroll
            for (int ks = 0; ks < kFK / 16; ++ks) {
                const uint64_t ad = tc::make_desc(a0 + ks * 2 * tc::kCoreBytes, tc::kCoreBytes, sbo_a);
                const uint64_t bd = tc::make_desc(P.sB[st] + ks * 2 * tc::kCoreBytes, tc::kCoreBytes, kFStage);
                tc::mma_bf16(P.tmem, ad, bd, P.idesc, (c > 0 || ks > 0) ? 1u : 0u);
            }
            tc::mma_commit(P.mbar[st]);
        }
    }
    // the loop waited for the MMAs of chunks 0 .. C - 3; wait for the last two
    for (int q = C >= 2 ? C - 2 : 0; q < C; ++q) {
        const int st = q & 1;
        const bool wt = tc::mbar_wait(P.mbar[st], P.par[st]);
        P.par[st] ^= 1u;
        ok = (__syncthreads_and(wt) != 0) && ok;
    }
    tc::fence_after_sync();
    return ok;
}

__global__ void __launch_bounds__(kFwdThreads, 2) k_mlp_forward(FeatParams fp, const float* __restrict__ xyt, int n,
                                                                 const bf16* __restrict__ wbf,
                                                                 const float* __restrict__ params,
                                                                 float* __restrict__ y, unsigned* err) {
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ __align__(8) uint64_t mbar[2];
    __shared__ uint32_t tmem_base;
    uint8_t* sB0 = smem;                 // weight stages: 2 x (256 rows x 32)
    uint8_t* sH = smem + 2 * 16384;      // activations: 4 K chunks of 128 x 64 (layer 0: feature stages)
    const int warp = threadIdx.x >> 5;
    const int row = threadIdx.x & 127;   // TMEM lane = ray of the tile (warp % 4 owns lanes 32 (warp % 4) ..)
    const int half = threadIdx.x >> 7;   // columns [128 half, 128 half + 128) of every layer
    if (warp == 0) tc::tmem_alloc(tc::smem_addr(&tmem_base), 256);
    if (threadIdx.x == 0) {
        tc::mbar_init(tc::smem_addr(&mbar[0]), 1);
        tc::mbar_init(tc::smem_addr(&mbar[1]), 1);
        tc::fence_mbar_init();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    FwdPipe P;
    P.sB[0] = tc::smem_addr(sB0);
    P.sB[1] = tc::smem_addr(sB0 + 16384);
    P.mbar[0] = tc::smem_addr(&mbar[0]);
    P.mbar[1] = tc::smem_addr(&mbar[1]);
    P.par[0] = P.par[1] = 0u;
    P.tmem = tmem_base;
    P.idesc = tc::make_idesc(kBM, kBN);
    const uint32_t lane_addr = tmem_base + ((uint32_t)((warp & 3) * 32) << 16);
    const uint32_t sHa = tc::smem_addr(sH);

    const int r = blockIdx.x * kBM + row;
    float u[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    const bool live = r < n;
    if (live) {
        float sn, cs;
        sincosf(__ldg(xyt + 3 * (size_t)r + 2), &sn, &cs);
        u[0] = __ldg(xyt + 3 * (size_t)r) * fp.inv_w;
        u[1] = __ldg(xyt + 3 * (size_t)r + 1) * fp.inv_h;
        u[2] = cs;
        u[3] = sn;
    }
    bool ok = fwd_layer<true>(P, wbf + w_offset(0), kFeat, sHa, sH, fp, u, live, row, half);
    for (int l = 0; l < kLayers && ok; ++l) {
        if (l > 0) ok = fwd_layer<false>(P, wbf + w_offset(l), kHidden, sHa, sH, fp, u, live, row, half);
        if (!ok) break;
        // epilogue of layer l: z = acc + b, rounded to bf16; h = bf16(GELU(z)) into sH
        const float* bias = params + b_offset(l);
        for (int cb = 128 * half; cb < 128 * half + 128; cb += 32) {
            float v[32];
            tc::tmem_ld32(lane_addr + cb, v);
#pragma unroll
            for (int i = 0; i < 32; i += 2) {
                const float z0 = v[i] + __ldg(bias + cb + i), z1 = v[i + 1] + __ldg(bias + cb + i + 1);
                const float2 zf = __bfloat1622float2(__floats2bfloat162_rn(z0, z1));
                *reinterpret_cast<__nv_bfloat162*>(sH + act_offset(row, cb + i)) =
                    __floats2bfloat162_rn(gelu(zf.x), gelu(zf.y));
            }
        }
        tc::fence_before_sync();   // TMEM reads done before the next layer's MMAs overwrite it
    }
    if (ok) {
        // output layer on the last activations, in k_out_layer's summation order: partial
        // sums over j = i (mod 32) in increasing j, then the xor butterfly
        __syncthreads();
        if (half == 0 && live) {
            const float* wout = params + kOutW;
            float part[32];
#pragma unroll
            for (int i = 0; i < 32; ++i) part[i] = 0.0f;
            for (int cb = 0; cb < kHidden; cb += 32) {
#pragma unroll
                for (int i = 0; i < 32; i += 8) {
                    const uint4 q = *reinterpret_cast<const uint4*>(sH + act_offset(row, cb + i));
                    const __nv_bfloat162* hb = reinterpret_cast<const __nv_bfloat162*>(&q);
#pragma unroll
                    for (int e = 0; e < 4; ++e) {
                        const float2 hf = __bfloat1622float2(hb[e]);
                        part[i + 2 * e] = __fadd_rn(part[i + 2 * e], __fmul_rn(hf.x, __ldg(wout + cb + i + 2 * e)));
                        part[i + 2 * e + 1] =
                            __fadd_rn(part[i + 2 * e + 1], __fmul_rn(hf.y, __ldg(wout + cb + i + 2 * e + 1)));
                    }
                }
            }
#pragma unroll
            for (int o = 16; o; o >>= 1)
#pragma unroll
                for (int i = 0; i < o; ++i) part[i] = __fadd_rn(part[i], part[i + o]);
            y[r] = __fadd_rn(part[0], __ldg(wout + kHidden));
        }
    } else if (threadIdx.x == 0) {
        atomicOr(err, 16u);
    }
    cp_async_wait<0>();
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(P.tmem, 256);
}

cudaError_t mlp_forward(const FeatParams& fp, const float* xyt, int n, const bf16* wbf, const float* params, float* y,
                        unsigned* err, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    static std::atomic<unsigned long long> attr{0};
    if (cudaError_t e = ensure_smem_attr(k_mlp_forward, (int)kFwdSmem, attr)) return e;
    k_mlp_forward<<<(n + kBM - 1) / kBM, kFwdThreads, kFwdSmem, s>>>(fp, xyt, n, wbf, params, y, err);
    return cudaGetLastError();
}

// output layer: y = H . w + b (fp32)
__global__ void k_out_layer(const bf16* __restrict__ H, const float* __restrict__ params, int n, float* __restrict__ y) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (warp >= n) return;
    const bf16* h = H + (size_t)warp * kHidden;
    const float* w = params + kOutW;
    float acc = 0.0f;
    for (int j = lane; j < kHidden; j += 32) acc += __bfloat162float(h[j]) * w[j];
    for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) y[warp] = acc + w[kHidden];
}

// --------------------------------------------------------------- training
// Huber loss (delta 1 px) against the target, mean over the batch; dy per ray.
__global__ void k_loss(const float* __restrict__ y, const float* __restrict__ t, int n, float* __restrict__ dy,
                       float* __restrict__ loss_sum) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    float l = 0.0f;
    if (r < n) {
        const float e = y[r] - t[r];
        const float ae = fabsf(e);
        l = ae <= 1.0f ? 0.5f * e * e : ae - 0.5f;
        dy[r] = (ae <= 1.0f ? e : copysignf(1.0f, e)) / (float)n;
    }
    for (int o = 16; o; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
    if ((threadIdx.x & 31) == 0 && l != 0.0f) atomicAdd(loss_sum, l);
}

// dZ of the last hidden layer = dy * w_out * GELU'(Z)
__global__ void k_out_backward(const float* __restrict__ dy, const bf16* __restrict__ Z,
                               const float* __restrict__ params, int n, bf16* __restrict__ dZ) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (warp >= n) return;
    const float g = dy[warp];
    const float* w = params + kOutW;
    for (int j = lane; j < kHidden; j += 32) {
        const size_t idx = (size_t)warp * kHidden + j;
        dZ[idx] = __float2bfloat16_rn(g * w[j] * gelu_grad(__bfloat162float(Z[idx])));
    }
}

// Column sums over rows of a [n x 256] bf16 matrix, each row weighted by w[r] (or 1): a block of
// 128 threads covers the 256 columns two per thread (one 4-byte load per row), its rows strided by
// the grid and four in flight per thread, then one atomic per column and block.
constexpr int kColSumBlocks = 4 * 152;
__device__ __forceinline__ void column_sums(const bf16* __restrict__ M, const float* __restrict__ w, int n,
                                            float* __restrict__ out, float* __restrict__ wsum) {
    const int c = 2 * threadIdx.x;
    float a0 = 0.0f, a1 = 0.0f, s = 0.0f;
    int r = blockIdx.x;
    for (; r + 3 * (int)gridDim.x < n; r += 4 * gridDim.x) {
        float2 v[4];
        float g[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int ru = r + u * gridDim.x;
            v[u] = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(M + (size_t)ru * kHidden + c));
            g[u] = w ? __ldg(w + ru) : 1.0f;
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            a0 += g[u] * v[u].x;
            a1 += g[u] * v[u].y;
            s += g[u];
        }
    }
    for (; r < n; r += gridDim.x) {
        const float2 v = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(M + (size_t)r * kHidden + c));
        const float g = w ? __ldg(w + r) : 1.0f;
        a0 += g * v.x;
        a1 += g * v.y;
        s += g;
    }
    atomicAdd(out + c, a0);
    atomicAdd(out + c + 1, a1);
    if (wsum && threadIdx.x == 0) atomicAdd(wsum, s);
}

// output-layer gradients: d w_out[j] = sum_r dy[r] H[r][j], d b_out = sum_r dy[r]
__global__ void __launch_bounds__(128) k_out_wgrad(const float* __restrict__ dy, const bf16* __restrict__ H, int n,
                                                   float* __restrict__ grads) {
    column_sums(H, dy, n, grads + kOutW, grads + kOutW + kHidden);
}

// column sums of dZ [n x 256] -> bias gradient
__global__ void __launch_bounds__(128) k_bias_grad(const bf16* __restrict__ dZ, int n, float* __restrict__ gb) {
    column_sums(dZ, nullptr, n, gb, nullptr);
}

// Adam (bias-corrected), fp32 master weights; refreshes the bf16 copies
__global__ void k_adam(float* __restrict__ p, float* __restrict__ m, float* __restrict__ v,
                       const float* __restrict__ g, size_t n, float lr, float b1, float b2, float eps, float c1,
                       float c2, bf16* __restrict__ wbf) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float pi = p[i] - lr * (mi * c1) / (sqrtf(vi * c2) + eps);
    p[i] = pi;
    wbf[i] = __float2bfloat16_rn(pi);
}

__global__ void k_to_bf16(const float* __restrict__ src, bf16* __restrict__ dst, size_t n) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = __float2bfloat16_rn(src[i]);
}

__device__ __forceinline__ uint32_t hash32(uint32_t x) {
    x ^= x >> 16; x *= 0x7feb352du; x ^= x >> 15; x *= 0x846ca68bu; x ^= x >> 16;
    return x;
}
__device__ __forceinline__ float u01(uint32_t a, uint32_t b) {
    return (hash32(a * 0x9e3779b9u ^ hash32(b)) >> 8) * (1.0f / 16777216.0f);
}

// uniform(-1/sqrt(fan_in), 1/sqrt(fan_in)) weights, zero biases, output bias = init_bias
__global__ void k_init_params(float* __restrict__ p, uint32_t seed, float init_bias) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kParamCount) return;
    float val = 0.0f;
    for (int l = 0; l < kLayers; ++l) {
        size_t w0 = w_offset(l), nw = (size_t)kHidden * layer_in(l);
        if (i >= w0 && i < w0 + nw) val = (2.0f * u01(seed, (uint32_t)i) - 1.0f) * rsqrtf((float)layer_in(l)) * 1.7f;
    }
    if (i >= kOutW && i < kOutW + kHidden) val = (2.0f * u01(seed, (uint32_t)i) - 1.0f) * rsqrtf((float)kHidden);
    if (i == kOutW + kHidden) val = init_bias;
    p[i] = val;
}

// ---------------------------------------------------- rays from the marcher
// The exact march (RangeLib.h:927-962) also reporting t at the hit step;
// t = max_range when the ray leaves the map or runs out of range.
__device__ float march_t(const MapDev& m, float mr, float x0, float y0, float c, float s, float* range) {
    float t = 0.0f;
    while (t < mr) {
        int px = __float2int_rz(__fadd_rn(x0, __fmul_rn(c, t)));
        int py = __float2int_rz(__fadd_rn(y0, __fmul_rn(s, t)));
        if ((unsigned)px >= (unsigned)m.W || (unsigned)py >= (unsigned)m.H) break;
        float d = __ldg(m.dt + (size_t)px * m.H + py);
        if (d <= 0.0f) {
            float xd = __fsub_rn(__int2float_rn(px), x0), yd = __fsub_rn(__int2float_rn(py), y0);
            *range = __fsqrt_rn(__fadd_rn(__fmul_rn(xd, xd), __fmul_rn(yd, yd)));
            return t;
        }
        t = __fadd_rn(t, fmaxf(__fmul_rn(d, 0.999f), 1.0f));
    }
    *range = mr;
    return mr;
}

// random free-cell poses, uniform heading; xyt (grid frame), t target, exact range
__global__ void k_sample_rays(MapDev m, float mr, const uint32_t* __restrict__ free_cells, uint32_t n_free,
                              uint32_t seed, long long base, int n, float* __restrict__ xyt, float* __restrict__ t,
                              float* __restrict__ range) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    const uint32_t id = (uint32_t)(base + r);
    const uint32_t cell = free_cells[hash32(id ^ hash32(seed)) % n_free];
    const int cx = (int)(cell / (uint32_t)m.H), cy = (int)(cell - (uint32_t)cx * (uint32_t)m.H);
    const float x = (float)cx + u01(id, seed ^ 0x1u), y = (float)cy + u01(id, seed ^ 0x2u);
    const float th = 6.2831853f * u01(id, seed ^ 0x3u);
    xyt[3 * (size_t)r] = x;
    xyt[3 * (size_t)r + 1] = y;
    xyt[3 * (size_t)r + 2] = th;
    float s, c, rg;
    rlc_trig::sincos_cr(th, &s, &c);   // the exact path's cos/sin
    t[r] = march_t(m, mr, x, y, c, s, &rg);
    if (range) range[r] = rg;
}

__global__ void k_free_flags(const uint64_t* __restrict__ bits, int W, int H, int TY, uint32_t* __restrict__ f) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)W * H) return;
    int x = (int)(i / H), y = (int)(i - (long long)x * H);
    uint64_t w = bits[(size_t)(x >> 3) * TY + (y >> 3)];
    f[i] = ((w >> (((x & 7) << 3) | (y & 7))) & 1ull) ? 0u : 1u;
}

__global__ void k_compact_free(const uint32_t* __restrict__ f, const uint32_t* __restrict__ pos, long long n,
                               uint32_t* __restrict__ out) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && f[i]) out[pos[i]] = (uint32_t)i;
}

// ------------------------------------------------------- learned inference
__device__ __forceinline__ bool occ_cell(const MapDev& m, int x, int y) {
    if ((unsigned)x >= (unsigned)m.W || (unsigned)y >= (unsigned)m.H) return false;
    uint64_t w = __ldg(m.bits + (size_t)(x >> 3) * m.tiles_y + (y >> 3));
    return (w >> (((x & 7) << 3) | (y & 7))) & 1ull;
}

// prediction -> accept check -> range (the reference's distance to the hit
// cell's corner); rejected rays are appended to the recast list
__global__ void k_accept(MapDev m, float mr, const float* __restrict__ xyt, const float* __restrict__ pred, int n,
                         float scale, float* __restrict__ outs, uint8_t* __restrict__ accepted,
                         int* __restrict__ recast, int* __restrict__ n_recast) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    const float x0 = xyt[3 * (size_t)r], y0 = xyt[3 * (size_t)r + 1], th = xyt[3 * (size_t)r + 2];
    const float t = pred[r];
    bool ok = false;
    float rg = 0.0f;
    if (t > 1.0f && t < 0.999f * mr && isfinite(t)) {
        float s, c;
        rlc_trig::sincos_cr(th, &s, &c);
        const int hx = __float2int_rz(x0 + c * t), hy = __float2int_rz(y0 + s * t);
        const int bx = __float2int_rz(x0 + c * (t - 1.0f)), by = __float2int_rz(y0 + s * (t - 1.0f));
        if (occ_cell(m, hx, hy) && !occ_cell(m, bx, by)) {
            const float xd = __fsub_rn(__int2float_rn(hx), x0), yd = __fsub_rn(__int2float_rn(hy), y0);
            rg = __fsqrt_rn(__fadd_rn(__fmul_rn(xd, xd), __fmul_rn(yd, yd)));
            ok = true;
        }
    }
    if (accepted) accepted[r] = ok ? 1 : 0;
    if (ok) {
        outs[r] = __fmul_rn(rg, scale);
    } else {
        int slot = atomicAdd(n_recast, 1);
        recast[slot] = r;
    }
}

__global__ void k_recast(MapDev m, float mr, const float* __restrict__ xyt, const int* __restrict__ list,
                         const int* __restrict__ count, float scale, float* __restrict__ outs) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= *count) return;
    const int r = list[j];
    const float x0 = xyt[3 * (size_t)r], y0 = xyt[3 * (size_t)r + 1], th = xyt[3 * (size_t)r + 2];
    float s, c, rg;
    rlc_trig::sincos_cr(th, &s, &c);
    march_t(m, mr, x0, y0, c, s, &rg);
    outs[r] = __fmul_rn(rg, scale);
}

// world-frame particles x beams -> grid-frame rays (RangeLib.h:482-520)
__global__ void k_world_rays(WorldDev w, const float* __restrict__ ins, const float* __restrict__ angles, int n,
                             int na, float* __restrict__ xyt) {
    long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= (long long)n * na) return;
    int i = (int)(g / na), a = (int)(g - (long long)i * na);
    float x = __fmul_rn(__fsub_rn(ins[3 * (size_t)i], w.ox), w.inv_s);
    float y = __fmul_rn(__fsub_rn(ins[3 * (size_t)i + 1], w.oy), w.inv_s);
    float tmp = x;
    x = __fsub_rn(__fmul_rn(w.ca, x), __fmul_rn(w.sa, y));
    y = __fadd_rn(__fmul_rn(w.sa, tmp), __fmul_rn(w.ca, y));
    const float th = __fsub_rn(__fadd_rn(-ins[3 * (size_t)i + 2], w.rc), angles[a]);
    xyt[3 * g] = y;   // calc_range(y, x, theta)
    xyt[3 * g + 1] = x;
    xyt[3 * g + 2] = th;
}

inline unsigned blocks_for(long long n, int b) { return (unsigned)((n + b - 1) / b); }

#define TRY(x) do { cudaError_t _e = (x); if (_e != cudaSuccess) return _e; } while (0)

}  // namespace

// ================================================================ host side
struct LearnedModel {
    MapDev map{};
    WorldDev world{};
    float mr = 0.0f;
    FeatParams fp{};
    float* params = nullptr;   // fp32 master [kParamCount]
    float* adam_m = nullptr;
    float* adam_v = nullptr;
    float* grads = nullptr;
    bf16* wbf = nullptr;       // bf16 copy of params (weights used by the GEMMs)
    unsigned* err = nullptr;
    long long adam_t = 0;
    // work buffers for a chunk of `cap` rays
    int cap = 0;
    bf16* X = nullptr;                 // [cap x 512]
    bf16* Z[kLayers] = {};             // pre-activations [cap x 256]
    bf16* Hh[kLayers] = {};            // activations
    bf16* dZ[2] = {};                  // ping-pong gradients
    // transposed copies, [column x cap]: the K-major operands of the weight-gradient GEMMs
    bf16* XT = nullptr;                // features [512 x cap]
    bf16* HT[kLayers - 1] = {};        // activations of layers 0-2 [256 x cap]
    bf16* dZT = nullptr;               // the current layer's gradient [256 x cap]
    bf16* wbfT = nullptr;              // weights of layers 1-3 transposed [in x out] (input gradients)
    float* y = nullptr;
    float* dy = nullptr;
    float* loss = nullptr;
    uint32_t* free_cells = nullptr;
    uint32_t n_free = 0;
    // query buffers (rays of one learned call)
    long long qcap = 0;
    float* q_xyt = nullptr;
    float* q_pred = nullptr;
    int* q_list = nullptr;
    int* q_cnt = nullptr;

    cudaError_t ensure_query(long long rays) {
        if (rays <= qcap) return cudaSuccess;
        cudaFree(q_xyt); cudaFree(q_pred); cudaFree(q_list); cudaFree(q_cnt);
        q_xyt = q_pred = nullptr; q_list = q_cnt = nullptr; qcap = 0;
        TRY(cudaMalloc(&q_xyt, (size_t)rays * 3 * sizeof(float)));
        TRY(cudaMalloc(&q_pred, (size_t)rays * sizeof(float)));
        TRY(cudaMalloc(&q_list, (size_t)rays * sizeof(int)));
        TRY(cudaMalloc(&q_cnt, sizeof(int)));
        qcap = rays;
        return cudaSuccess;
    }

    void free_work() {
        cudaFree(X);
        for (int l = 0; l < kLayers; ++l) { cudaFree(Z[l]); cudaFree(Hh[l]); Z[l] = Hh[l] = nullptr; }
        cudaFree(dZ[0]); cudaFree(dZ[1]);
        cudaFree(XT); cudaFree(dZT); cudaFree(wbfT);
        for (int l = 0; l < kLayers - 1; ++l) { cudaFree(HT[l]); HT[l] = nullptr; }
        cudaFree(y); cudaFree(dy); cudaFree(loss);
        X = nullptr; dZ[0] = dZ[1] = nullptr; y = dy = loss = nullptr;
        XT = dZT = wbfT = nullptr;
        cap = 0;
    }
    ~LearnedModel() {
        free_work();
        cudaFree(params); cudaFree(adam_m); cudaFree(adam_v); cudaFree(grads); cudaFree(wbf); cudaFree(err);
        cudaFree(free_cells);
        cudaFree(q_xyt); cudaFree(q_pred); cudaFree(q_list); cudaFree(q_cnt);
    }
    cudaError_t ensure(int rows) {
        rows = (rows + kBM - 1) / kBM * kBM;
        if (rows <= cap) return cudaSuccess;
        free_work();
        TRY(cudaMalloc(&X, (size_t)rows * kFeat * sizeof(bf16)));
        for (int l = 0; l < kLayers; ++l) {
            TRY(cudaMalloc(&Z[l], (size_t)rows * kHidden * sizeof(bf16)));
            TRY(cudaMalloc(&Hh[l], (size_t)rows * kHidden * sizeof(bf16)));
        }
        TRY(cudaMalloc(&dZ[0], (size_t)rows * kHidden * sizeof(bf16)));
        TRY(cudaMalloc(&dZ[1], (size_t)rows * kHidden * sizeof(bf16)));
        TRY(cudaMalloc(&XT, (size_t)rows * kFeat * sizeof(bf16)));
        for (int l = 0; l < kLayers - 1; ++l) TRY(cudaMalloc(&HT[l], (size_t)rows * kHidden * sizeof(bf16)));
        TRY(cudaMalloc(&dZT, (size_t)rows * kHidden * sizeof(bf16)));
        TRY(cudaMalloc(&wbfT, (size_t)(kLayers - 1) * kWh * sizeof(bf16)));
        TRY(cudaMalloc(&y, (size_t)rows * sizeof(float)));
        TRY(cudaMalloc(&dy, (size_t)rows * sizeof(float)));
        TRY(cudaMalloc(&loss, sizeof(float)));
        cap = rows;
        return cudaSuccess;
    }

    // K split of the weight-gradient GEMMs: chunks of >= 256 rows, at most 64 splits
    static int split_k(int rows) {
        int sp = rows;
        for (int parts = 64; parts > 1; parts >>= 1)
            if (rows % (parts * 256) == 0) { sp = rows / parts; break; }
        return sp;
    }

    GemmArgs base_args() const {
        GemmArgs g{};
        g.err = err;
        return g;
    }

    // forward over `rows` rays whose features are in X; predictions in y
    cudaError_t forward(int rows, cudaStream_t s) {
        const bf16* in = X;
        for (int l = 0; l < kLayers; ++l) {
            GemmArgs g = base_args();
            g.A = in; g.lda = layer_in(l); g.a_t = 0;
            g.B = wbf + w_offset(l); g.ldb = layer_in(l); g.b_t = 0;   // W [out x in]: N x K, K-major
            g.M = rows; g.N = kHidden; g.K = layer_in(l);
            g.epi = EPI_FWD; g.ldc = kHidden;
            g.bias = params + b_offset(l);
            g.Zout = Z[l]; g.Hout = Hh[l];
            if (l < kLayers - 1) { g.HoutT = HT[l]; g.ldt = cap; }
            TRY(gemm(g, s));
            in = Hh[l];
        }
        k_out_layer<<<blocks_for((long long)rows * 32, 256), 256, 0, s>>>(Hh[kLayers - 1], params, rows, y);
        return cudaGetLastError();
    }

    // backward from dy (rows rays, features in X, forward state in Z/Hh); gradients into grads
    cudaError_t backward(int rows, cudaStream_t s) {
        TRY(cudaMemsetAsync(grads, 0, kParamCount * sizeof(float), s));
        k_out_backward<<<blocks_for((long long)rows * 32, 256), 256, 0, s>>>(dy, Z[kLayers - 1], params, rows, dZ[0]);
        TRY(cudaGetLastError());
        k_out_wgrad<<<kColSumBlocks, 128, 0, s>>>(dy, Hh[kLayers - 1], rows, grads);
        TRY(cudaGetLastError());
        // K-major operands of the weight and input gradients: features and the top gradient
        // transposed here, the hidden activations by the forward epilogue, the weights of layers 1-3
        TRY(transpose_bf16(X, rows, kFeat, kFeat, XT, cap, s));
        TRY(transpose_bf16(dZ[0], rows, kHidden, kHidden, dZT, cap, s));
        for (int l = 1; l < kLayers; ++l)
            TRY(transpose_bf16(wbf + w_offset(l), kHidden, kHidden, kHidden, wbfT + (size_t)(l - 1) * kWh, kHidden, s));
        int cur = 0;
        for (int l = kLayers - 1; l >= 0; --l) {
            // weight gradient: dW [out x in] = dZ^T . input  (K = rows)
            GemmArgs gw = base_args();
            gw.A = dZT; gw.lda = cap;                               // A[m=out][k=row] = dZ[row][out]
            gw.B = l == 0 ? XT : HT[l - 1]; gw.ldb = cap;           // B[n=in][k=row] = input[row][in]
            gw.M = kHidden; gw.N = layer_in(l); gw.K = rows;
            gw.ksplit = split_k(rows);                              // split the batch across CTAs
            gw.epi = EPI_F32_ADD; gw.ldc = layer_in(l); gw.C32 = grads + w_offset(l);
            TRY(gemm(gw, s));
            k_bias_grad<<<kColSumBlocks, 128, 0, s>>>(dZ[cur], rows, grads + b_offset(l));
            TRY(cudaGetLastError());
            if (l == 0) break;
            // input gradient: dH = dZ . W, then times GELU'(Z[l-1])
            GemmArgs gx = base_args();
            gx.A = dZ[cur]; gx.lda = kHidden;                       // A[m=row][k=out]
            gx.B = wbfT + (size_t)(l - 1) * kWh; gx.ldb = kHidden;  // B[n=in][k=out] = W[out][in]
            gx.M = rows; gx.N = layer_in(l); gx.K = kHidden;
            gx.epi = EPI_BWD; gx.ldc = kHidden;
            gx.Zin = Z[l - 1]; gx.dZ = dZ[cur ^ 1];
            gx.dZT = dZT; gx.ldt = cap;                             // the next layer's weight-gradient operand
            TRY(gemm(gx, s));
            cur ^= 1;
        }
        return cudaSuccess;
    }

    cudaError_t features(const float* xyt, int n, cudaStream_t s) {
        const int rows = (n + kBM - 1) / kBM * kBM;
        k_features<<<blocks_for(rows, 128), 128, 0, s>>>(fp, xyt, n, rows, X);
        return cudaGetLastError();
    }

    cudaError_t adam_step(float lr, cudaStream_t s) {
        ++adam_t;
        const float b1 = 0.9f, b2 = 0.999f;
        const float c1 = 1.0f / (1.0f - powf(b1, (float)adam_t)), c2 = 1.0f / (1.0f - powf(b2, (float)adam_t));
        k_adam<<<blocks_for((long long)kParamCount, 256), 256, 0, s>>>(params, adam_m, adam_v, grads, kParamCount, lr,
                                                                      b1, b2, 1e-8f, c1, c2, wbf);
        return cudaGetLastError();
    }
};

}  // namespace rlc

// ======================================================================= ABI
using namespace rlc;

struct rlc_learned {
    LearnedModel m;
};

namespace {
char g_msg[512];
int lfail(int code, const char* what, cudaError_t e = cudaSuccess) {
    if (e != cudaSuccess) snprintf(g_msg, sizeof(g_msg), "%s: %s", what, cudaGetErrorString(e));
    else snprintf(g_msg, sizeof(g_msg), "%s", what);
    return set_last_error(code, g_msg);
}
#define LTRY(expr, what) do { cudaError_t _e = (expr); if (_e != cudaSuccess) return lfail(RLC_ERR_CUDA, what, _e); } while (0)
}  // namespace

extern "C" {

int rlc_learned_create(const rlc_method* rm, unsigned seed, rlc_learned** out) {
    if (!out) return lfail(RLC_ERR_ARG, "null output handle");
    *out = nullptr;
    MapDev map;
    WorldDev world;
    float mr;
    if (int rc = method_map_view(rm, &map, &world, &mr)) return rc;
    rlc_learned* L = new rlc_learned();
    LearnedModel& M = L->m;
    M.map = map;
    M.world = world;
    M.mr = mr;
    M.fp.inv_w = 1.0f / (float)map.W;
    M.fp.inv_h = 1.0f / (float)map.H;
    const double fmax = std::max(2.0, 0.5 * std::max(map.W, map.H));
    for (int k = 0; k < 64; ++k) M.fp.freq[k] = (float)std::pow(fmax, k / 63.0);
    cudaError_t e = cudaSuccess;
    if (e == cudaSuccess) e = cudaMalloc(&M.params, kParamCount * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&M.adam_m, kParamCount * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&M.adam_v, kParamCount * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&M.grads, kParamCount * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&M.wbf, kParamCount * sizeof(bf16));
    if (e == cudaSuccess) e = cudaMalloc(&M.err, sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMemset(M.err, 0, sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMemset(M.adam_m, 0, kParamCount * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(M.adam_v, 0, kParamCount * sizeof(float));
    if (e == cudaSuccess) {
        k_init_params<<<blocks_for((long long)kParamCount, 256), 256>>>(M.params, seed, 0.25f * mr);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
        k_to_bf16<<<blocks_for((long long)kParamCount, 256), 256>>>(M.params, M.wbf, kParamCount);
        e = cudaGetLastError();
    }
    // free cells of the map, for sampling training rays
    if (e == cudaSuccess) {
        const long long n = (long long)map.W * map.H;
        uint32_t *f = nullptr, *pos = nullptr;
        e = cudaMalloc(&f, (n + 1) * sizeof(uint32_t));
        if (e == cudaSuccess) e = cudaMalloc(&pos, (n + 1) * sizeof(uint32_t));
        if (e == cudaSuccess) {
            k_free_flags<<<blocks_for(n, 256), 256>>>(map.bits, map.W, map.H, map.tiles_y, f);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = scan_exclusive_u32(f, pos, (size_t)n, 0);
        if (e == cudaSuccess) e = cudaMemcpy(&M.n_free, pos + n, sizeof(uint32_t), cudaMemcpyDeviceToHost);
        if (e == cudaSuccess) e = cudaMalloc(&M.free_cells, (size_t)(M.n_free ? M.n_free : 1) * sizeof(uint32_t));
        if (e == cudaSuccess) {
            k_compact_free<<<blocks_for(n, 256), 256>>>(f, pos, n, M.free_cells);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = cudaDeviceSynchronize();
        cudaFree(f);
        cudaFree(pos);
    }
    if (e != cudaSuccess) {
        delete L;
        return lfail(RLC_ERR_CUDA, "learned model setup", e);
    }
    if (M.n_free == 0) {
        delete L;
        return lfail(RLC_ERR_ARG, "the map has no free cell to sample rays from");
    }
    *out = L;
    return RLC_OK;
}

int rlc_learned_destroy(rlc_learned* L) {
    delete L;
    return RLC_OK;
}

int64_t rlc_learned_param_count(void) { return (int64_t)kParamCount; }

int rlc_learned_get_params(rlc_learned* L, float* host_params) {
    if (!L || !host_params) return lfail(RLC_ERR_ARG, "null argument");
    LTRY(cudaMemcpy(host_params, L->m.params, kParamCount * sizeof(float), cudaMemcpyDeviceToHost), "get params");
    return RLC_OK;
}

int rlc_learned_set_params(rlc_learned* L, const float* host_params) {
    if (!L || !host_params) return lfail(RLC_ERR_ARG, "null argument");
    LTRY(cudaMemcpy(L->m.params, host_params, kParamCount * sizeof(float), cudaMemcpyHostToDevice), "set params");
    k_to_bf16<<<blocks_for((long long)kParamCount, 256), 256>>>(L->m.params, L->m.wbf, kParamCount);
    LTRY(cudaGetLastError(), "set params");
    LTRY(cudaMemset(L->m.adam_m, 0, kParamCount * sizeof(float)), "set params");
    LTRY(cudaMemset(L->m.adam_v, 0, kParamCount * sizeof(float)), "set params");
    L->m.adam_t = 0;
    return RLC_OK;
}

// Sample rays from the map's free cells with the exact marcher (device buffers, n rays).
int rlc_learned_sample_rays(rlc_learned* L, long long first_id, unsigned seed, int n, float* d_xyt, float* d_t,
                            float* d_range, void* stream) {
    if (!L || n < 0 || (n > 0 && (!d_xyt || !d_t))) return lfail(RLC_ERR_ARG, "bad argument");
    if (n == 0) return RLC_OK;
    LearnedModel& M = L->m;
    k_sample_rays<<<blocks_for(n, 256), 256, 0, (cudaStream_t)stream>>>(M.map, M.mr, M.free_cells, M.n_free, seed,
                                                                        first_id, n, d_xyt, d_t, d_range);
    LTRY(cudaGetLastError(), "sample rays");
    return RLC_OK;
}

// Forward only: predicted t for n grid-frame rays (device buffers).
int rlc_learned_predict(rlc_learned* L, const float* d_xyt, int n, float* d_pred, void* stream) {
    if (!L || n < 0 || (n > 0 && (!d_xyt || !d_pred))) return lfail(RLC_ERR_ARG, "bad argument");
    LearnedModel& M = L->m;
    LTRY(mlp_forward(M.fp, d_xyt, n, M.wbf, M.params, d_pred, M.err, (cudaStream_t)stream), "fused forward");
    return RLC_OK;
}

// The same predictions through the training path's layer-by-layer GEMMs (test reference).
int rlc_learned_predict_layered(rlc_learned* L, const float* d_xyt, int n, float* d_pred, void* stream) {
    if (!L || n < 0 || (n > 0 && (!d_xyt || !d_pred))) return lfail(RLC_ERR_ARG, "bad argument");
    LearnedModel& M = L->m;
    cudaStream_t s = (cudaStream_t)stream;
    const int chunk = 262144;
    LTRY(M.ensure(std::min(n, chunk)), "predict buffers");
    for (int off = 0; off < n; off += chunk) {
        const int cnt = std::min(chunk, n - off);
        const int rows = (cnt + kBM - 1) / kBM * kBM;
        LTRY(M.features(d_xyt + 3 * (size_t)off, cnt, s), "features");
        LTRY(M.forward(rows, s), "forward");
        LTRY(cudaMemcpyAsync(d_pred + off, M.y, cnt * sizeof(float), cudaMemcpyDeviceToDevice, s), "predict");
    }
    return RLC_OK;
}

// Test hook: the bf16 features of n grid-frame rays into d_out [n x 512] (device).
int rlc_learned_features(rlc_learned* L, const float* d_xyt, int n, void* d_out) {
    if (!L || n <= 0 || !d_xyt || !d_out) return lfail(RLC_ERR_ARG, "bad argument");
    k_features<<<blocks_for(n, 128), 128>>>(L->m.fp, d_xyt, n, n, (bf16*)d_out);
    LTRY(cudaGetLastError(), "features");
    LTRY(cudaDeviceSynchronize(), "features");
    return RLC_OK;
}

// One forward + backward over n rays (device buffers) without an update:
// host_grads receives the parameter gradients of the mean Huber loss.
int rlc_learned_gradients(rlc_learned* L, const float* d_xyt, const float* d_t, int n, float* host_grads,
                          float* host_loss) {
    if (!L || n <= 0 || !d_xyt || !d_t) return lfail(RLC_ERR_ARG, "bad argument");
    if (n % kBM) return lfail(RLC_ERR_ARG, "gradients take a multiple of 128 rays");
    LearnedModel& M = L->m;
    LTRY(M.ensure(n), "gradient buffers");
    LTRY(M.features(d_xyt, n, 0), "features");
    LTRY(M.forward(n, 0), "forward");
    LTRY(cudaMemset(M.loss, 0, sizeof(float)), "loss");
    k_loss<<<blocks_for(n, 256), 256>>>(M.y, d_t, n, M.dy, M.loss);
    LTRY(cudaGetLastError(), "loss");
    LTRY(M.backward(n, 0), "backward");
    LTRY(cudaDeviceSynchronize(), "gradients");
    unsigned err = 0;
    LTRY(cudaMemcpy(&err, M.err, sizeof(unsigned), cudaMemcpyDeviceToHost), "gradients");
    if (err) return lfail(RLC_ERR_CUDA, "tensor-core GEMM timed out waiting for its MMAs");
    if (host_grads) LTRY(cudaMemcpy(host_grads, M.grads, kParamCount * sizeof(float), cudaMemcpyDeviceToHost), "grads");
    if (host_loss) {
        float l = 0.0f;
        LTRY(cudaMemcpy(&l, M.loss, sizeof(float), cudaMemcpyDeviceToHost), "loss");
        *host_loss = l / (float)n;
    }
    return RLC_OK;
}

// Train on rays drawn by the exact marcher: `steps` Adam steps of `batch` rays
// (a multiple of 128), cosine-decayed learning rate from lr.  *final_loss gets
// the mean loss of the last 20 steps.
int rlc_learned_train(rlc_learned* L, int steps, int batch, float lr, unsigned seed, float* final_loss,
                      void* stream) {
    if (!L || steps < 0 || batch <= 0 || batch % kBM) return lfail(RLC_ERR_ARG, "batch must be a positive multiple of 128");
    LearnedModel& M = L->m;
    cudaStream_t s = (cudaStream_t)stream;
    LTRY(M.ensure(batch), "train buffers");
    float *xyt = nullptr, *tt = nullptr;
    LTRY(cudaMalloc(&xyt, (size_t)batch * 3 * sizeof(float)), "train buffers");
    cudaError_t e = cudaMalloc(&tt, (size_t)batch * sizeof(float));
    float loss_acc = 0.0f;
    int loss_n = 0;
    for (int st = 0; st < steps && e == cudaSuccess; ++st) {
        k_sample_rays<<<blocks_for(batch, 256), 256, 0, s>>>(M.map, M.mr, M.free_cells, M.n_free, seed,
                                                             (long long)st * batch, batch, xyt, tt, nullptr);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = M.features(xyt, batch, s);
        if (e == cudaSuccess) e = M.forward(batch, s);
        if (e == cudaSuccess) e = cudaMemsetAsync(M.loss, 0, sizeof(float), s);
        if (e == cudaSuccess) {
            k_loss<<<blocks_for(batch, 256), 256, 0, s>>>(M.y, tt, batch, M.dy, M.loss);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = M.backward(batch, s);
        const float cosine = 0.5f * (1.0f + cosf(3.14159265f * (float)st / (float)(steps > 1 ? steps : 1)));
        if (e == cudaSuccess) e = M.adam_step(lr * (0.05f + 0.95f * cosine), s);
        if (e == cudaSuccess && st >= steps - 20) {
            float l = 0.0f;
            e = cudaMemcpyAsync(&l, M.loss, sizeof(float), cudaMemcpyDeviceToHost, s);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s);
            loss_acc += l / (float)batch;
            ++loss_n;
        }
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(xyt);
    cudaFree(tt);
    if (e != cudaSuccess) return lfail(RLC_ERR_CUDA, "training", e);
    unsigned err = 0;
    LTRY(cudaMemcpy(&err, M.err, sizeof(unsigned), cudaMemcpyDeviceToHost), "training");
    if (err) return lfail(RLC_ERR_CUDA, "tensor-core GEMM timed out waiting for its MMAs");
    if (final_loss) *final_loss = loss_n ? loss_acc / loss_n : 0.0f;
    return RLC_OK;
}

// Learned calc_range_repeat_angles (world frame, device buffers): predicted
// hit cells that pass the check give the reference's corner distance, the
// rest are recast exactly.  accepted (optional) marks accepted rays; *n_recast
// gets the number of recast rays.
int rlc_learned_calc_range_repeat_angles(rlc_learned* L, const float* d_ins, const float* d_angles, float* d_outs,
                                         int n, int na, uint8_t* d_accepted, int64_t* n_recast, void* stream) {
    if (!L || n < 0 || na < 0) return lfail(RLC_ERR_ARG, "bad argument");
    const long long rays = (long long)n * na;
    if (rays == 0) return RLC_OK;
    if (!d_ins || !d_angles || !d_outs) return lfail(RLC_ERR_ARG, "null array");
    if (rays > (1ll << 31) - 1) return lfail(RLC_ERR_ARG, "too many rays");
    LearnedModel& M = L->m;
    cudaStream_t s = (cudaStream_t)stream;
    LTRY(M.ensure_query(rays), "learned query buffers");
    float* xyt = M.q_xyt;
    float* pred = M.q_pred;
    int* list = M.q_list;
    int* cnt = M.q_cnt;
    cudaError_t e = cudaMemsetAsync(cnt, 0, sizeof(int), s);
    if (e == cudaSuccess) {
        k_world_rays<<<blocks_for(rays, 256), 256, 0, s>>>(M.world, d_ins, d_angles, n, na, xyt);
        e = cudaGetLastError();
    }
    int rc = RLC_OK;
    if (e == cudaSuccess) rc = rlc_learned_predict(L, xyt, (int)rays, pred, stream);
    if (e == cudaSuccess && !rc) {
        k_accept<<<blocks_for(rays, 256), 256, 0, s>>>(M.map, M.mr, xyt, pred, (int)rays, M.world.s, d_outs,
                                                       d_accepted, list, cnt);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess && !rc) {
        k_recast<<<blocks_for(rays, 256), 256, 0, s>>>(M.map, M.mr, xyt, list, cnt, M.world.s, d_outs);
        e = cudaGetLastError();
    }
    int h_cnt = 0;
    if (e == cudaSuccess && !rc) e = cudaMemcpyAsync(&h_cnt, cnt, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess && !rc) e = cudaStreamSynchronize(s);
    if (rc) return rc;
    if (e != cudaSuccess) return lfail(RLC_ERR_CUDA, "learned ranges", e);
    if (n_recast) *n_recast = h_cnt;
    return RLC_OK;
}

// Test hook: C[M x N] (fp32, row-major) = A . B^T on the tensor cores, with A
// [M x K] (or K x M when a_t) and B [N x K] (or K x N when b_t), bf16, device.
int rlc_tc_gemm(const void* d_a, const void* d_b, float* d_c, int M, int N, int K, int a_t, int b_t, void* stream) {
    if (!d_a || !d_b || !d_c) return lfail(RLC_ERR_ARG, "null pointer");
    if (M <= 0 || N <= 0 || K <= 0 || M % kBM || N % kBN || K % tc::kKChunk)
        return lfail(RLC_ERR_ARG, "M must be a multiple of 128, N of 256, K of 64");
    unsigned* err = nullptr;
    bf16 *at = nullptr, *bt = nullptr;   // K-major copies of transposed operands
    const cudaStream_t s = (cudaStream_t)stream;
    LTRY(cudaMalloc(&err, sizeof(unsigned)), "gemm");
    cudaError_t e = cudaMemset(err, 0, sizeof(unsigned));
    GemmArgs g{};
    g.A = (const bf16*)d_a; g.lda = K;
    g.B = (const bf16*)d_b; g.ldb = K;
    if (e == cudaSuccess && a_t) {   // A given as [K x M]
        e = cudaMalloc(&at, (size_t)M * K * sizeof(bf16));
        if (e == cudaSuccess) e = transpose_bf16((const bf16*)d_a, K, M, M, at, K, s);
        g.A = at;
    }
    if (e == cudaSuccess && b_t) {   // B given as [K x N]
        e = cudaMalloc(&bt, (size_t)N * K * sizeof(bf16));
        if (e == cudaSuccess) e = transpose_bf16((const bf16*)d_b, K, N, N, bt, K, s);
        g.B = bt;
    }
    g.M = M; g.N = N; g.K = K;
    g.epi = EPI_F32; g.ldc = N; g.C32 = d_c; g.err = err;
    if (e == cudaSuccess) e = gemm(g, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    unsigned h = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&h, err, sizeof(unsigned), cudaMemcpyDeviceToHost);
    cudaFree(err);
    cudaFree(at);
    cudaFree(bt);
    if (e != cudaSuccess) return lfail(RLC_ERR_CUDA, "tensor-core gemm", e);
    if (h) return lfail(RLC_ERR_CUDA, "tensor-core GEMM timed out waiting for its MMAs");
    return RLC_OK;
}

}  // extern "C"
