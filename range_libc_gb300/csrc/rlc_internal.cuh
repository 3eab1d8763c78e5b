// Internal device structures and kernel launchers of the GB300 ray-casting
// library.  Everything here is private to librangelibc_gb300.so; the public
// surface is include/rangelibc.h.
//
// Grid layout: the occupancy grid and the distance transform index cells as
// (x, y) with x < width, y < height -- the reference's OMap::grid[x][y].
//   * occupancy: 8x8 bit tiles, one uint64 per tile, tiles x-major;
//     bit ((x & 7) << 3 | (y & 7)) of word (x >> 3) * tiles_y + (y >> 3).
//   * distance transform: float, either linear x-major (x * height + y,
//     the reference's kernels.cu:15-17 layout) or 8x8 tiles of 64 floats
//     (256 B, two 128-B lines) in the same tile order; or the compact form:
//     the integer squared distance d^2 as uint16 in 8x8 tiles of 128 B whose
//     four 32-B sectors hold 4x4 cells each, 0xFFFF meaning "d^2 >= 65535,
//     read the float".  Every DT value is sqrtf of an integer below 2^24, so
//     sqrtf(d^2) reproduces it exactly.
#pragma once

#include <cuda_runtime.h>

#include "rlc_trig.cuh"

#include <atomic>
#include <stdint.h>

struct rlc_method;

namespace rlc {

enum Kind : int { K_BL = 0, K_RM = 1, K_CDDT = 2, K_GLT = 3 };

// error flags a kernel can raise (ORed into a per-method device word)
enum DevFlag : unsigned {
    F_BL_BOUND = 1u,       // Bresenham loop bound reached (coordinates beyond float's integer range)
    F_WRAP_BOUND = 2u,     // CDDT heading wrap loop bound reached (|heading| > ~6e5 rad)
    F_CDDT_PAST_END = 4u,  // forward binary search with x equal to the last zero point
    F_NAN_INDEX = 8u,      // NaN range/observation mapped to sensor bin 0
};

enum DtLayout : int { DT_LINEAR = 0, DT_TILED = 1, DT_U16 = 2, DT_STAGED = 3, DT_STEP = 4, DT_RUNS = 5 };

struct MapDev {
    int W, H;
    int tiles_y;              // ceil(H / 8)
    const float* dt;          // distance transform (DT_LINEAR / DT_TILED; linear for DT_U16)
    const uint16_t* dt16;     // compact squared distances (DT_U16)
    const uint8_t* dt8;       // 8-bit squared distances (DT_STAGED windows)
    const float* step;        // march step per cell, max(dt * 0.999, 1), 0 on occupied cells (DT_STEP, DT_RUNS)
    // DT_RUNS: per cell, how many consecutive cells after it have the same step value, along +y,
    // -y, +x and -x (bits 0-7, 8-15, 16-23, 24-31; at most 255)
    const uint32_t* runs;
    const uint64_t* bits;     // occupancy bit tiles
};

struct CddtDev {
    unsigned td;
    float td_div_2pi;         // theta_discretization / M_2PI, as float
    float twopi_div_td;       // M_2PI / theta_discretization, as float
    const int* widths;        // [td]
    const float* trans;       // [td]
    const float* cosv;        // [td] cosf of each discrete angle (host libm)
    const float* sinv;        // [td]
    const uint32_t* slice_base;  // [td + 1]
    const uint32_t* bin_start;   // [total_bins + 1]
    const float* zeros;
};

// GiantLUTCast table (RangeLib.h:1772-1904): lut[(x * H + y) * td + i]
struct GltDev {
    const uint16_t* lut;
    unsigned td;
    float td_div_2pi;         // theta_discretization / M_2PI, as float
    float max_div_limits;     // max_range / 65535
};

struct WorldDev {
    float inv_s, s, rc, ox, oy, sa, ca;
};

struct CastParams {
    int kind;
    float mr;
    MapDev map;
    CddtDev cddt;
    GltDev glt;
    WorldDev world;
    const float* trig;        // optional per-ray (cos, sin) override (parity mode)
    unsigned* err;            // device error word
};

struct SensorDev {
    const double* table;      // K x K row-major, table[r * K + d]
    int K;
};

// ---- map preprocessing (rlc_map.cu) ----
cudaError_t launch_pack_bits(const uint8_t* d_occ, int W, int H, uint64_t* d_bits, cudaStream_t s);
cudaError_t launch_edt(const uint64_t* d_bits, int W, int H, int tiles_y, float* d_dt_linear,
                       void* scratch, size_t scratch_bytes, cudaStream_t s);
size_t edt_scratch_bytes(int W, int H);
// upper bound of edt_scratch_bytes(W, H) over all W * H <= cells with W, H <= side
constexpr size_t edt_scratch_bound(size_t cells, size_t side) {
    return ((cells * 4 + 255) & ~(size_t)255) + cells * 4 + (cells + side) * 8 + 256;
}
cudaError_t launch_dt_to_tiled(const float* d_lin, int W, int H, float* d_tiled, cudaStream_t s);
cudaError_t launch_dt_to_u16(const float* d_lin, int W, int H, uint16_t* d_u16, cudaStream_t s);
// the ray-marching step of every cell (linear layout), as RayMarching::calc_range forms it
cudaError_t launch_dt_to_step(const float* d_lin, int W, int H, float* d_step, cudaStream_t s);
// equal-step run lengths of the step map along both axes (MapDev::runs)
cudaError_t launch_step_runs(const float* d_step, int W, int H, uint32_t* d_runs, cudaStream_t s);
cudaError_t launch_dt_to_u8(const float* d_lin, int W, int H, uint8_t* d_u8, cudaStream_t s);
cudaError_t launch_edge_map(const uint64_t* d_bits, int W, int H, int tiles_y, uint8_t* d_edge, cudaStream_t s);
cudaError_t launch_unpack_bits(const uint64_t* d_bits, int W, int H, int tiles_y, uint8_t* d_occ, cudaStream_t s);

// ---- casting (rlc_cast.cu) ----
// layout: DtLayout of the distance transform; pf: 1 = RM prefetching schedule
cudaError_t launch_calc_range_many(const CastParams& p, int layout, int pf, bool world, const float* ins,
                                   float* outs, int n, cudaStream_t s);
cudaError_t launch_repeat_angles(const CastParams& p, int layout, int pf, const float* ins, const float* angles,
                                 float* outs, int n, int na, cudaStream_t s);
cudaError_t launch_eval_sensor(const CastParams& p, const SensorDev& sm, const float* obs,
                               const float* ranges, double* outs, int na, int n, cudaStream_t s);
// block: threads per block (0 = 256); tile: particles per tile (0 = auto)
cudaError_t launch_fused(const CastParams& p, int layout, int pf, const SensorDev& sm, const float* ins,
                         const float* angles, const float* obs, double* weights, int n, int na,
                         int block, int tile, cudaStream_t s);
// particles per tile the fused kernel uses
int tile_particles(int na, int block, int tile);

// beam-major fused particle update with a staged shared-memory window of the
// 8-bit distance transform (RM only): bins[a * n + i] receives each ray's
// range bin, then the per-particle products run in a second kernel.
// The grid is beams x chunks blocks of the particles; chunks = 0 picks
// max(1, SMs / beams) so that the grid fills the GPU once.
cudaError_t launch_fused_staged(const CastParams& p, const SensorDev& sm, const float* ins, const float* angles,
                                const float* obs, double* weights, int n, int na, int chunks,
                                uint16_t* bins, cudaStream_t s);

// GiantLUTCast construction: one ray march (linear DT, the given per-angle
// cos/sin) from every cell corner at every angle bin, clamped to max_range
// and stored as uint16 (RangeLib.h:1782-1818)
cudaError_t launch_glt_build(const MapDev& map, float mr, unsigned td, const float* cosv, const float* sinv,
                             float limits_div_max, uint16_t* lut, cudaStream_t s);
// CDDT calc_range_pair of one grid-frame query (RangeLib.h:1521-1615): out[0] = r, out[1] = r_inv
cudaError_t launch_cddt_pair(const CastParams& p, float x, float y, float heading, float* out, cudaStream_t s);
// calc_range_many_radial_optimized (RangeLib.h:616-676) for world-frame poses:
// beam a < max(mp + 1, off) at heading offset angles[a]; see k_cddt_radial
cudaError_t launch_cddt_radial(const CastParams& p, const float* ins, const float* angles, float* outs, int n,
                               int num_rays, int mp, int off, cudaStream_t s);

// march steps of world-frame repeat-angle rays (RM and BL), summed into *total
cudaError_t launch_count_steps(const CastParams& p, const float* ins, const float* angles, int n, int na,
                               unsigned long long* total, cudaStream_t s);

// sincos[2i], sincos[2i + 1] = the casts' sin and cos of x[i] (rlc_trig::sincos_cr)
cudaError_t launch_trig_eval(const float* x, float* sincos, long long n, cudaStream_t s);

// ---- batched multi-filter update (rlc_cast.cu) ----
struct FilterDev {
    CastParams p;
    int layout;
    int prefetch;
    SensorDev sm;
    const float* ins;
    const float* angles;
    const float* obs;
    float* ranges;            // optional pixel ranges
    double* weights;
    uint16_t* bins;           // range bins (batch scratch), per tile beam-major in groups of 4 beams
    uint16_t* obs_bins;       // na observation bins (batch scratch, written at the start of each run)
    // ray-marching batches (batch scratch, written at the start of each run): per particle two
    // float4, {x, y, heading} in the grid frame and the heading's sin and cos as float pairs
    // {sin hi, sin lo, cos hi, cos lo}; per beam the angle's sin and cos as float pairs.  A NaN
    // sin hi marks a value without pairs (its rays compute their cos/sin directly).
    float4* part_rec;
    float4* beam_rec;
    int n, na, ppb;           // particles, beams, particles per tile
    float inv_na;             // 1 / (float)na rounded to nearest (tile ray -> particle, beam)
    unsigned tile_begin;      // first global tile of this filter
    unsigned part_begin;      // first global particle of this filter
};
// Range bins of a batch tile: ceil(na / 4) groups x ppb particles x 4 beams, so that a lane
// reads a particle's four bins of one group with one 8-byte load; tiles follow one another.
__host__ __device__ inline size_t batch_tile_bins(int na, int ppb) { return (size_t)((na + 3) >> 2) * ppb * 4; }
__host__ __device__ inline size_t batch_tile_offset(const FilterDev& F, int tile) {
    return (size_t)tile * batch_tile_bins(F.na, F.ppb);
}
// cudaFuncSetAttribute(MaxDynamicSharedMemorySize) of `kernel` once per device (the attribute
// belongs to the device's context); `done` holds one bit per device already set.
template <class K>
inline cudaError_t ensure_smem_attr(K kernel, int bytes, std::atomic<unsigned long long>& done) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const unsigned long long bit = dev < 64 ? 1ull << dev : 0ull;
    if (bit && (done.load(std::memory_order_acquire) & bit)) return cudaSuccess;
    e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess && bit) done.fetch_or(bit, std::memory_order_release);
    return e;
}

// Bytes of a CDDT zero-point array of nz entries: whole 32-byte sectors, so that the bin search
// may read the full sector around any entry (bound_s).
inline size_t cddt_zeros_bytes(size_t nz) { return ((nz + 7) / 8 + (nz == 0)) * 8 * sizeof(float); }
// Persistent launch: `grid` blocks of `block` threads draw tiles from *queue
// (which must be zero) until all `total_tiles` are done.  rm_only selects the
// kernel specialised for batches whose filters all ray-march, with the
// distance-transform layout and prefetch given; otherwise every filter's own
// kind, layout and prefetch are dispatched at run time.  The per-particle
// products run overlapped inside the persistent kernel, or (separate) in a
// second launch over all `total_particles` after the cast.
cudaError_t launch_batch(const FilterDev* d_filters, int nf, unsigned total_tiles, unsigned* queue, int grid,
                         int block, size_t smem, bool rm_only, int layout, int pf, bool separate,
                         unsigned total_particles, cudaStream_t s);
// dynamic shared memory of a batch launch (the ray-marching kernel's per-warp slots of handed-on rays)
size_t batch_smem(int block, bool rm_only);
cudaError_t batch_occupancy(int block, size_t smem, bool rm_only, int layout, int pf, bool separate,
                            int* blocks_per_sm);

// ---- CDDT table (rlc_cddt.cu) ----
struct CddtBuild {
    uint32_t* slice_base = nullptr;   // device [td + 1]
    uint32_t* bin_start = nullptr;    // device [total_bins + 1]
    float* zeros = nullptr;           // device
    uint32_t total_bins = 0;
    uint32_t nzeros = 0;
};
// Builds the table on the device; widths/trans/cos/sin are device arrays of td entries,
// h_slice_base the host copy of the per-slice bin offsets.
cudaError_t cddt_build(const uint64_t* d_bits, int W, int H, int tiles_y, unsigned td,
                       const int* d_widths, const float* d_trans, const float* d_cos, const float* d_sin,
                       const uint32_t* h_slice_base, CddtBuild* out, cudaStream_t s, char* why, size_t why_len);
cudaError_t cddt_prune(const uint64_t* d_bits, int W, int H, int tiles_y, unsigned td, float max_range,
                       const int* d_widths, const float* d_trans, const float* d_cos, const float* d_sin,
                       CddtBuild* tab, cudaStream_t s);

// the device view of a ray-marching method's map (linear DT), world frame and
// max_range; RLC_ERR_* on a null or non-RM method (rlc_api.cu)
int method_map_view(const struct ::rlc_method* m, MapDev* map, WorldDev* world, float* max_range);

// ---- error reporting (rlc_api.cu) ----
// records `msg` as the calling thread's rlc_last_error() text and returns `code`
int set_last_error(int code, const char* msg);

// ---- utilities (rlc_cddt.cu) ----
// exclusive scan of n uint32 values; d_out[n] receives the total.
cudaError_t scan_exclusive_u32(const uint32_t* d_in, uint32_t* d_out, size_t n, cudaStream_t s);

}  // namespace rlc
