/*
 * rangelibc.h -- C ABI of the GB300 (sm_103a) ray-casting library.
 *
 * Drop-in boundary for range_libc's batched hot path (kctess5/range_libc).
 * Every entry point below replaces one method of the reference's C++
 * `ranges::RangeMethod` family (includes/RangeLib.h) or of its CUDA helper
 * `RayMarchingCUDA` (includes/CudaRangeLib.h, includes/kernels.cu); the
 * citation is given beside each declaration.  The C++ classes of
 * include/RangeLib.h and the Python module range_libc_gb300.range_libc are
 * thin layers over these functions.
 *
 * Conventions
 *  - Status: every function returns RLC_OK (0) or an RLC_ERR_* code, and
 *    rlc_last_error() gives a message for the calling thread.  Nothing
 *    throws across the ABI.
 *  - Grid layout: occ[x * height + y] != 0 marks cell (x, y) occupied, x <
 *    width, y < height (the reference's OMap::grid[x][y]).
 *  - Pointers: by default every array argument is HOST memory and the call is
 *    synchronous (results are in place on return), like the reference.  With
 *    RLC_DEVICE_PTRS every array argument is DEVICE memory and the call is
 *    asynchronous on `stream` (NULL = the legacy default stream).
 *  - World frame: calls without RLC_NO_WORLD apply the reference's ROS
 *    world->grid transform (RangeLib.h:439-480): scale, rotate, then
 *    calc_range(y, x, theta) with theta = -theta_world - world_angle - 3*pi/2,
 *    and ranges multiplied by world_scale.
 *  - Array layouts: poses ins[n][3] = (x, y, theta) float32; angles[na];
 *    ranges of repeat-angle calls are particle-major outs[i * na + a];
 *    sensor tables are K x K float64 row-major, table[r * K + d].
 *  - A map's occupancy is immutable once created; methods share its device
 *    data (reference-counted, so a map may be destroyed before its methods)
 *    and copy its world parameters at creation, so like the reference's
 *    methods (which take OMap by value) they do not see later
 *    rlc_map_set_world calls.  A method handle must not be used by two host
 *    threads at once.
 *  - No CPU fallback: with no usable GPU every call returns RLC_ERR_CUDA.
 */
#ifndef RANGELIBC_H
#define RANGELIBC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define RLC_API __attribute__((visibility("default")))
#else
#define RLC_API
#endif

#define RLC_ABI_VERSION 1

typedef struct rlc_map rlc_map;
typedef struct rlc_method rlc_method;
typedef struct rlc_batch rlc_batch;

enum rlc_status {
    RLC_OK = 0,
    RLC_ERR_ARG = 1,      /* invalid argument (null pointer, size, kind) */
    RLC_ERR_CUDA = 2,     /* CUDA runtime error (message in rlc_last_error) */
    RLC_ERR_STATE = 3,    /* call not valid in the handle's state (e.g. no sensor model) */
    RLC_ERR_NOMEM = 4,    /* device allocation failed */
    RLC_ERR_IO = 5        /* a file could not be read, decoded or written */
};

enum rlc_kind {
    RLC_BL = 0,           /* BresenhamsLine,   RangeLib.h:691-772 */
    RLC_RM = 1,           /* RayMarching,      RangeLib.h:922-969 */
    RLC_CDDT = 2,         /* CDDTCast,         RangeLib.h:971-1770 */
    RLC_PCDDT = 3,        /* CDDTCast + prune(max_range) (PyCDDTCast + prune, RangeLibc.pyx:253-262) */
    RLC_RMGPU = 4,        /* RayMarchingGPU,   RangeLib.h:774-920 (same kernels as RLC_RM) */
    RLC_GLT = 5           /* GiantLUTCast,     RangeLib.h:1772-1904 (16-bit table built on the device) */
};

enum rlc_flags {
    RLC_DEVICE_PTRS = 1u, /* array arguments are device pointers; asynchronous on `stream` */
    RLC_NO_WORLD = 2u     /* calc_range_many only: raw calc_range(x, y, theta) per row, no
                             world transform (RayMarchingGPU::calc_range_many, RangeLib.h:835-846) */
};

/* kernel-reported conditions, read with rlc_method_device_flags */
enum rlc_device_flag {
    RLC_FLAG_BL_BOUND = 1u,       /* Bresenham loop bound hit by a walk that has not yet passed the
                                     grid's far edge: a start beyond 2^24 where float +-1 no longer
                                     moves it, or a walk that skips its end cell where float +-1
                                     rounds up across a power of two.  (A walk past the grid's edge in
                                     its direction of motion ends there with max_range, unflagged.) */
    RLC_FLAG_WRAP_BOUND = 2u,     /* CDDT heading wrap bound hit (|heading| > ~6e5 rad) */
    RLC_FLAG_CDDT_PAST_END = 4u,  /* query equal to a bin's last zero point (reference reads past the bin) */
    RLC_FLAG_NAN_INDEX = 8u       /* NaN range or observation mapped to sensor bin 0 */
};

/* ---- library ---------------------------------------------------------- */
RLC_API int rlc_abi_version(void);
RLC_API const char* rlc_last_error(void);
/* Number of CUDA devices visible (0 when none); never fails. */
RLC_API int rlc_device_count(void);

/* ---- maps: OMap (RangeLib.h:121-322) ---------------------------------- */
/* OMap(int w, int h) + grid fill (RangeLib.h:143-156; PyOMap(ndarray), RangeLibc.pyx:140-145). */
RLC_API int rlc_map_create(const uint8_t* occ, int width, int height, rlc_map** out);
/* OMap(std::string filename, float threshold) (RangeLib.h:158-201): the PNG's pixel (x, y) is
 * occupied when (int)rgb2gray(r, g, b) < threshold, with r, g, b the pixel's blue, green and red
 * (the reference reads bytes 2, 1, 0 of each RGBA pixel).  Host code, no GPU.  Call with
 * occ = NULL to read width and height; then again with those and occ[width * height] to get
 * occ[x * height + y].  Non-interlaced PNGs of every colour type and bit depth; RLC_ERR_IO with
 * the reason in rlc_last_error() for files that cannot be read or decoded. */
RLC_API int rlc_png_occupancy(const char* path, float threshold, uint8_t* occ, int* width, int* height);
/* OMap::save (RangeLib.h:263-291): occ[x * height + y] as an 8-bit grey PNG, occupied black and
 * free white.  Host code, no GPU. */
RLC_API int rlc_png_save_occupancy(const char* path, const uint8_t* occ, int width, int height);
/* World parameters of the ROS conversion (RangeLib.h:134-141; RangeLibc.pyx:160-180). */
RLC_API int rlc_map_set_world(rlc_map* map, float scale, float angle, float origin_x, float origin_y,
                              float sin_angle, float cos_angle);
RLC_API int rlc_map_destroy(rlc_map* map);
/* OMap::width/height (RangeLibc.pyx:191-197). */
RLC_API int rlc_map_size(const rlc_map* map, int* width, int* height);
/* OMap::grid export (host, occ[x * height + y]). */
RLC_API int rlc_map_occupancy(rlc_map* map, uint8_t* occ_out);
/* DistanceTransform(OMap*) (RangeLib.h:345-373), computed on the device; host export. */
RLC_API int rlc_map_distance_transform(rlc_map* map, float* dt_out);
/* OMap::make_edge_map(true) (RangeLib.h:293-312); host export. */
RLC_API int rlc_map_edge_map(rlc_map* map, uint8_t* edge_out);

/* ---- range methods ----------------------------------------------------- */
/* BresenhamsLine(OMap, mr) / RayMarching(OMap, mr) / CDDTCast(OMap, mr, td) /
 * RayMarchingGPU(OMap, mr) / GiantLUTCast(OMap, mr, td) constructors.  theta_disc is used by
 * CDDT and GLT only.  The CDDT table and the GLT table (width x height x td uint16: one ray
 * march from every cell corner at every angle bin, RangeLib.h:1782-1818) are built on the
 * device. */
RLC_API int rlc_method_create(rlc_map* map, int kind, float max_range, unsigned theta_disc, rlc_method** out);
/* CDDT constructor with caller-supplied cosines and sines of the td discrete
 * angles i * (2*pi/td) (as float).  Used to pin a table to another host's libm. */
RLC_API int rlc_method_create_cddt_trig(rlc_map* map, int kind, float max_range, unsigned theta_disc,
                                        const float* cos_tab, const float* sin_tab, rlc_method** out);
RLC_API int rlc_method_destroy(rlc_method* m);
RLC_API int rlc_method_info(const rlc_method* m, int* kind, float* max_range, unsigned* theta_disc);
/* Kernel-reported conditions since the last call (see rlc_device_flag); clears them. */
RLC_API int rlc_method_device_flags(rlc_method* m, unsigned* flags);

/* CDDTCast::prune(float max_range) (RangeLib.h:1176-1283), on the device. */
RLC_API int rlc_cddt_prune(rlc_method* m, float max_range);
/* CDDT table access (compressed_lut, lut_translations; RangeLib.h:1742-1748). */
RLC_API int rlc_cddt_table_size(rlc_method* m, int64_t* num_bins, int64_t* num_zeros);
RLC_API int rlc_cddt_table_export(rlc_method* m, int* widths, float* trans, int64_t* bin_len, float* zeros);
/* Replace the table (same theta_disc and bin counts), e.g. one exported from the reference. */
RLC_API int rlc_cddt_table_load(rlc_method* m, const float* trans, const int64_t* bin_len, const float* zeros,
                                int64_t num_zeros);

/* GiantLUTCast table export: lut[(x * height + y) * td + i] as the reference stores it
 * (giant_lut[x][y][i], RangeLib.h:1782-1818). */
RLC_API int rlc_glt_table(rlc_method* m, uint16_t* lut_out);

/* CDDTCast::calc_range_pair(x, y, heading) (RangeLib.h:1521-1615): the ranges at heading and
 * at heading + pi from one bin search, in grid space.  A bin outside the slice gives
 * (max_range, max_range) where the reference indexes it unchecked. */
RLC_API int rlc_cddt_calc_range_pair(rlc_method* m, float x, float y, float heading, float* r, float* r_inv);
/* CDDTCast::calc_range_many_radial_optimized(ins, outs, n, num_rays, min_angle, max_angle)
 * (RangeLib.h:616-676): world-frame poses, num_rays beams from min_angle to max_angle, the
 * first num_rays/3 beams cast in pairs with the beam pi further on.  Positions of a row the
 * reference does not write keep the caller's values; writes the reference sends past a
 * particle's row are dropped (the next particle overwrites them there). */
RLC_API int rlc_cddt_calc_range_many_radial(rlc_method* m, const float* ins, float* outs, int n, int num_rays,
                                            float min_angle, float max_angle, unsigned flags, void* stream);

/* Host buffers of calls without RLC_DEVICE_PTRS.  RLC_HOST_AUTO (default): where the GPU reads
 * and writes pageable host memory coherently (Grace + Blackwell over NVLink-C2C,
 * cudaDevAttrPageableMemoryAccess) the kernels work on the caller's buffers in place; elsewhere
 * the buffers are staged through device memory.  RLC_HOST_STAGED: always stage.  Process-wide. */
enum rlc_host_path_mode { RLC_HOST_AUTO = 0, RLC_HOST_STAGED = 1 };
RLC_API int rlc_set_host_path(int mode);
/* 1 if host-pointer calls on the current device run in place, 0 if they are staged. */
RLC_API int rlc_host_path(int* direct);

/* ---- queries ----------------------------------------------------------- */
/* RangeMethod::calc_range(x, y, heading) (virtual, RangeLib.h:419): one ray in grid space. */
RLC_API int rlc_calc_range(rlc_method* m, float x, float y, float heading, float* out);
/* RangeMethod::numpy_calc_range (RangeLib.h:439-480; RayMarchingCUDA::numpy_calc_range,
 * kernels.cu:245-260).  With RLC_NO_WORLD: RayMarchingGPU::calc_range_many (kernels.cu:232-243). */
RLC_API int rlc_calc_range_many(rlc_method* m, const float* ins, float* outs, int n, unsigned flags,
                                void* stream);
/* RangeMethod::numpy_calc_range_angles (RangeLib.h:482-520; kernels.cu:263-279). */
RLC_API int rlc_calc_range_repeat_angles(rlc_method* m, const float* ins, const float* angles, float* outs,
                                         int n, int num_angles, unsigned flags, void* stream);
/* RangeMethod::set_sensor_model (RangeLib.h:523-532; RayMarchingCUDA::set_sensor_table, kernels.cu:224-229). */
RLC_API int rlc_set_sensor_model(rlc_method* m, const double* table, int table_width);
/* RangeMethod::eval_sensor_model (RangeLib.h:533-555). */
RLC_API int rlc_eval_sensor_model(rlc_method* m, const float* obs, const float* ranges, double* outs,
                                  int rays_per_particle, int particles, unsigned flags, void* stream);
/* RangeMethod::calc_range_repeat_angles_eval_sensor_model (RangeLib.h:558-612); fused on the
 * device, replacing the unimplemented RayMarchingCUDA version (kernels.cu:281-315). */
RLC_API int rlc_calc_range_repeat_angles_eval_sensor_model(rlc_method* m, const float* ins,
                                                           const float* angles, const float* obs,
                                                           double* weights, int n, int num_angles,
                                                           unsigned flags, void* stream);

/* Parity mode (testing): per-ray (cos, sin) pairs, ray-indexed like the outputs of the
 * next query calls (BL and RM).  trig = NULL restores the device's own (rlc_trig_eval).  `count` rays,
 * host pointer; the array is copied. */
RLC_API int rlc_method_set_trig_override(rlc_method* m, const float* trig, int64_t count);

/* The cos/sin the BL and RM casts use for a ray heading x when no trig override is set: the
 * floats nearest to the exact sin(x) and cos(x) (the reference calls the host libm's sinf/cosf,
 * RangeLib.h:700-702, 930-931, which glibc rounds to nearest on all but ~0.1 % of arguments).
 * sincos[2 i] = sin(x[i]), sincos[2 i + 1] = cos(x[i]), computed by the device; with
 * RLC_DEVICE_PTRS both arrays are device memory and the call is queued on `stream`.  Lets a
 * checker reproduce the production casts bit for bit. */
RLC_API int rlc_trig_eval(const float* x, float* sincos, int64_t n, unsigned flags, void* stream);

/* Measurement: total march steps of the rays of a repeat-angle call (RM: distance-transform
 * reads; BL: cells tested), for stating algorithmic bytes.  Synchronous; RM and BL only. */
RLC_API int rlc_count_steps(rlc_method* m, const float* ins, const float* angles, int n, int num_angles,
                            unsigned flags, int64_t* total_steps);

/* ---- tuning ------------------------------------------------------------ */
/* Schedule of the kernels: dt_layout 0 = linear x-major distance transform, 1 = 8x8 tiles,
 * 2 = compact 16-bit squared distances, 4 = linear map of each cell's march step
 * max(d * 0.999, 1) (0 on occupied cells), 5 = that step map plus, per cell, how many cells after
 * it along each axis have the same step, so that a ray repeating one step beside a wall (6 times
 * in a row) skips the rest of the run in one go (exactly: the skipped steps' parameters are formed by the reference's own float
 * additions and the landing cell is checked), 3 = beam-major fused update that stages each bundle's
 * window of 8-bit squared distances in shared memory (RM only; tile = particle chunks per beam,
 * 0 = one block per SM) (-1 = autotune on the next fused call); fused_block = threads per block of the fused kernel
 * (0 = keep); prefetch 1 = prefetch the distance transform ahead of each RM ray; for CDDT
 * methods prefetch selects the bin search: 0 binary, 1 warp-cooperative (32 zero points per
 * step, ballot; calc_range_many and calc_range_repeat_angles), 2 by 32-byte sectors for bins of
 * more than 32 zero points (fewer dependent reads; pays when queries spread over the map); tile =
 * particles per tile of the fused and batched kernels (0 = automatic).  Results are identical
 * under every schedule. */
RLC_API int rlc_method_set_schedule(rlc_method* m, int dt_layout, int fused_block, int prefetch, int tile);
RLC_API int rlc_method_get_schedule(const rlc_method* m, int* dt_layout, int* fused_block, int* prefetch,
                                    int* tile);
/* Time the schedule candidates on a workload (device pointers) and keep the fastest: the median
 * of 5 single launches for every candidate, then the median of 31 for the three fastest, taken
 * round-robin.  rlc_method_autotune_ex with RLC_TUNE_FLUSH_L2 writes twice the L2 size before
 * every timed launch (for callers whose maps leave L2 between updates; it holds that buffer for
 * the call), and rlc_method_autotune_results returns the candidates of the last autotune:
 * schedules[4 i .. 4 i + 3] = (dt_layout, fused_block, prefetch, tile) and times_ms[2 i],
 * times_ms[2 i + 1] = first-stage and final medians (0 when not a finalist); at most `max`
 * entries are written, *count gets the number of candidates. */
enum rlc_tune_flags { RLC_TUNE_FLUSH_L2 = 1u };
RLC_API int rlc_method_autotune(rlc_method* m, const float* d_ins, const float* d_angles, const float* d_obs,
                                double* d_weights, int n, int num_angles, void* stream);
RLC_API int rlc_method_autotune_ex(rlc_method* m, const float* d_ins, const float* d_angles, const float* d_obs,
                                   double* d_weights, int n, int num_angles, unsigned flags, void* stream);
RLC_API int rlc_method_autotune_results(const rlc_method* m, int max, int* count, int* schedules, float* times_ms);

/* ---- distance transform without device allocation ----------------------------
 * No counterpart in the reference.  For callers that may not call cudaMalloc (real-time
 * loops that forbid allocation after start-up; hosts whose device memory belongs to another
 * allocator): computes the same distance transform as rlc_map_distance_transform from a
 * device occupancy grid d_occ[x * height + y] (uint8, != 0 occupied) into device memory
 * d_dt[x * height + y] (float), asynchronously on `stream`, allocating nothing.  Its
 * scratch is a fixed device array of RLC_NOALLOC_SCRATCH_BYTES that every GPU loading this
 * library holds until exit; maps beyond RLC_NOALLOC_MAX_CELLS cells or RLC_NOALLOC_MAX_SIDE
 * per side are rejected with RLC_ERR_ARG, and so are pointers that are not device memory of the
 * current device (or managed memory).  The first call on a device looks up the array's
 * address there and keeps it (make it before any stream capture; after cudaDeviceReset,
 * reload the library before calling again).  Calls share the array: calls that overlap on the
 * GPU race and corrupt each other's results. */
#define RLC_NOALLOC_MAX_CELLS 1048576
#define RLC_NOALLOC_MAX_SIDE 4096
#define RLC_NOALLOC_SCRATCH_BYTES 16949760
RLC_API int rlc_distance_transform_noalloc(const uint8_t* d_occ, int width, int height, float* d_dt,
                                           void* stream);

/* ---- batched multi-filter particle update (no reference counterpart) --------
 * Many independent filters, each a method (RM or BL or CDDT) with its own map, poses,
 * beams, observation and sensor table, run as one persistent launch that draws
 * particle tiles from a device queue; rlc_batch_run replays it as a CUDA graph. */
typedef struct rlc_filter_desc {
    rlc_method* method;   /* sensor model must be set */
    const float* ins;     /* device [n_particles][3] world poses */
    const float* angles;  /* device [n_angles] */
    const float* obs;     /* device [n_angles] world ranges */
    float* ranges;        /* device [n_particles * n_angles] pixel ranges, or NULL */
    double* weights;      /* device [n_particles] */
    int n_particles;
    int n_angles;
} rlc_filter_desc;

/* The methods must outlive the batch.  block = threads per block (0 = 256).  A method's trig
 * override set or cleared after the batch was created is taken up by the next rlc_batch_run. */
RLC_API int rlc_batch_create(const rlc_filter_desc* filters, int n_filters, int block, rlc_batch** out);
RLC_API int rlc_batch_run(rlc_batch* b, void* stream);
/* Schedule of the persistent launch: distance-transform layout (0 linear, 1 tiled, 2 compact
 * 16-bit, 4 step map, 5 step map with equal-step runs) and prefetch of every ray-marching filter,
 * threads per block, particles per tile
 * (0 = 32).  Results are identical under every schedule. */
RLC_API int rlc_batch_set_schedule(rlc_batch* b, int dt_layout, int prefetch, int block, int tile);
RLC_API int rlc_batch_get_schedule(const rlc_batch* b, int* dt_layout, int* prefetch, int* block, int* tile);
/* Where the per-particle products run: RLC_PRODUCTS_OVERLAPPED -- inside the persistent kernel,
 * warp 0 of a block multiplying its previous tile while the other warps cast the next one;
 * RLC_PRODUCTS_SEPARATE -- in a second launch over all particles after the cast (both in the
 * graph).  Weights are identical; rlc_batch_autotune picks the faster. */
enum rlc_product_mode { RLC_PRODUCTS_OVERLAPPED = 0, RLC_PRODUCTS_SEPARATE = 1 };
RLC_API int rlc_batch_set_product_mode(rlc_batch* b, int mode);
RLC_API int rlc_batch_get_product_mode(const rlc_batch* b, int* mode);
/* Run the batch under each schedule candidate on `stream` and keep the fastest. */
RLC_API int rlc_batch_autotune(rlc_batch* b, void* stream);
RLC_API int rlc_batch_destroy(rlc_batch* b);
/* rays = sum of n_particles * n_angles; tiles = work items of the device queue */
RLC_API int rlc_batch_info(const rlc_batch* b, int64_t* rays, int64_t* tiles);

/* ---- learned range surrogate (no reference counterpart) ----------------------
 * A per-map MLP (512 Fourier features of x/W, y/H, cos, sin -> 4 x 256 GELU -> 1) predicting
 * where a ray reaches its hit cell, trained on the GPU (tcgen05 BF16 GEMMs, FP32 accumulation,
 * Adam) on rays cast by the exact ray marcher of an RM method.  Queries accept a prediction
 * whose cell is occupied while the cell one pixel before is free, returning the reference's
 * distance to that cell's corner; every other ray is recast exactly.  Device pointers. */
typedef struct rlc_learned rlc_learned;
RLC_API int rlc_learned_create(const rlc_method* ray_marching, unsigned seed, rlc_learned** out);
RLC_API int rlc_learned_destroy(rlc_learned* l);
RLC_API int64_t rlc_learned_param_count(void);
RLC_API int rlc_learned_get_params(rlc_learned* l, float* host_params);
RLC_API int rlc_learned_set_params(rlc_learned* l, const float* host_params);
/* n rays from uniform free-cell poses: grid-frame (x, y, theta) [n][3], hit parameter t, exact range */
RLC_API int rlc_learned_sample_rays(rlc_learned* l, long long first_id, unsigned seed, int n, float* d_xyt,
                                    float* d_t, float* d_range, void* stream);
RLC_API int rlc_learned_train(rlc_learned* l, int steps, int batch, float lr, unsigned seed, float* final_loss,
                              void* stream);
/* t of n grid-frame rays by the fused forward kernel (the whole network per 128-ray tile on one SM) */
RLC_API int rlc_learned_predict(rlc_learned* l, const float* d_xyt, int n, float* d_pred, void* stream);
/* the same through the layer-by-layer GEMMs of the training path (bit-identical; test reference) */
RLC_API int rlc_learned_predict_layered(rlc_learned* l, const float* d_xyt, int n, float* d_pred, void* stream);
RLC_API int rlc_learned_calc_range_repeat_angles(rlc_learned* l, const float* d_ins, const float* d_angles,
                                                 float* d_outs, int n, int num_angles, uint8_t* d_accepted,
                                                 int64_t* n_recast, void* stream);
/* testing: features of grid-frame rays (bf16 [n][512]); gradients of the mean Huber loss over n
 * (a multiple of 128) rays into host_grads [rlc_learned_param_count()]; a tensor-core GEMM
 * C[M x N] = A . B^T (bf16 in, fp32 out; A is K x M when a_t, B is K x N when b_t). */
RLC_API int rlc_learned_features(rlc_learned* l, const float* d_xyt, int n, void* d_out);
RLC_API int rlc_learned_gradients(rlc_learned* l, const float* d_xyt, const float* d_t, int n, float* host_grads,
                                  float* host_loss);
RLC_API int rlc_tc_gemm(const void* d_a, const void* d_b, float* d_c, int M, int N, int K, int a_t, int b_t,
                        void* stream);

#ifdef __cplusplus
}
#endif
#endif /* RANGELIBC_H */
