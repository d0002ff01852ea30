/*
 * dsmvc_gb300: C ABI of the GB300 (sm_103a) descale executor.
 *
 * The drop-in boundary for the reference's `backend="cuda"` path.  The
 * VapourSynth plugin shim, the tests, the benchmark and the request loop all
 * call these functions.  Plain C types only: no C++ or torch types cross this
 * boundary.  Every function returns DSMVC_GB_OK (0) or an error code;
 * dsmvc_gb_last_error() returns the calling thread's last message.  The
 * reference reports the same conditions as C++ exceptions:
 *   invalid_argument   -> DSMVC_GB_INVALID_ARGUMENT
 *   runtime_error      -> DSMVC_GB_RUNTIME_ERROR (incl. Float64 NaN/inf)
 *   length_error, out_of_range -> DSMVC_GB_LENGTH_ERROR
 * (src/vs_plugin.cpp:1748-1757 turns them into setFilterError).
 *
 * Strides are in samples.  Host buffers may be exactly
 * (rows - 1) * stride + width samples; row padding beyond the logical width
 * is never read or written (include/dsmvc/engine.hpp:231-235).
 */
#ifndef DSMVC_GB300_H
#define DSMVC_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DSMVC_GB_ABI_VERSION 1

enum dsmvc_gb_status {
    DSMVC_GB_OK = 0,
    DSMVC_GB_INVALID_ARGUMENT = 1,
    DSMVC_GB_RUNTIME_ERROR = 2,
    DSMVC_GB_LENGTH_ERROR = 3,
    DSMVC_GB_CUDA_ERROR = 4,
    DSMVC_GB_OUT_OF_MEMORY = 5,
    DSMVC_GB_UNAVAILABLE = 6
};

/* KernelKind, BorderMode, F64Mode: include/dsmvc/engine.hpp:16-60. */
enum dsmvc_gb_kernel_kind {
    DSMVC_GB_BILINEAR = 0, DSMVC_GB_BICUBIC = 1, DSMVC_GB_LANCZOS = 2,
    DSMVC_GB_SPLINE16 = 3, DSMVC_GB_SPLINE36 = 4, DSMVC_GB_SPLINE64 = 5,
    DSMVC_GB_CUSTOM = 6
};
enum dsmvc_gb_border {
    DSMVC_GB_ZERO = 0, DSMVC_GB_REPEAT = 1, DSMVC_GB_REFLECT101 = 2,
    DSMVC_GB_SYMMETRIC = 3, DSMVC_GB_MIRROR = 4
};
enum dsmvc_gb_f64_mode {
    DSMVC_GB_F64_AUTO = 0, DSMVC_GB_F64_OFF = 1, DSMVC_GB_F64_FORCE = 2
};
enum dsmvc_gb_sample {
    DSMVC_GB_FLOAT32 = 0, DSMVC_GB_UINT8 = 1, DSMVC_GB_UINT16 = 2
};

/* AxisRequest + KernelSpec (include/dsmvc/engine.hpp:62-76). */
typedef struct dsmvc_gb_axis_request {
    int32_t source_size;
    int32_t destination_size;
    double active_length;
    double shift;
    int32_t kernel;          /* enum dsmvc_gb_kernel_kind */
    int32_t taps;
    double b;
    double c;
    double blur;
    int32_t border;          /* enum dsmvc_gb_border */
    int32_t f64_mode;        /* enum dsmvc_gb_f64_mode */
} dsmvc_gb_axis_request;

/* IntegerConversion (include/dsmvc/engine.hpp:167-173); 20 bytes like the
 * reference's IntegerConversionDescriptor (src/cuda/cuda_kernel.hpp:20-26). */
typedef struct dsmvc_gb_conversion {
    float input_offset;
    float input_scale;
    float output_scale;
    float output_offset;
    uint32_t output_maximum;
} dsmvc_gb_conversion;

/* Read-only summary of a plan (AxisPlan scalars, engine.hpp:82-138). */
typedef struct dsmvc_gb_plan_info {
    int32_t source_size;
    int32_t destination_size;
    int32_t support;
    int32_t half_bandwidth;
    int32_t requires_float64;
    int32_t max_row_entries;
    double active_length;
    double shift;
    double normal_rcond;
    double normal_inf_norm;
    uint64_t nonzeros;
    uint64_t storage_bytes;
} dsmvc_gb_plan_info;

typedef struct dsmvc_gb_planner_stats {
    uint64_t plan_hits;
    uint64_t plan_builds;
    uint64_t plan_entries;
    uint64_t plan_resident_bytes;
} dsmvc_gb_planner_stats;

/* Executor counters.  The plan cache holds device copies of plans that were
 * not prepared (an LRU keyed by plan identity, DSMVC_GB_PLAN_CACHE_MB =
 * 16..4096 MiB, default 2048; the reference's packed-plan cache,
 * src/cuda/cuda_executor.cpp:1936-2020, DSMVC_CUDA_PLAN_CACHE_MB). */
typedef struct dsmvc_gb_executor_stats {
    uint64_t launches;
    uint64_t plane_tasks;
    uint64_t plan_uploads;
    uint64_t device_plan_bytes;
    uint64_t workspace_bytes;
    uint64_t plan_cache_hits;
    uint64_t plan_cache_misses;
    uint64_t plan_cache_evictions;
    uint64_t plan_cache_bytes;
    uint64_t compile_reuses;      /* calls that reused their slot's compiled launches */
} dsmvc_gb_executor_stats;

/* One plane of a device-resident batch.  `horizontal`/`vertical` may be
 * NULL for a one-axis descale (then `vectors` is the row or column count). */
typedef struct dsmvc_gb_plan dsmvc_gb_plan;
typedef struct dsmvc_gb_plane_task {
    const dsmvc_gb_plan *horizontal;
    const dsmvc_gb_plan *vertical;
    const void *input;            /* device pointer */
    int64_t input_stride;         /* samples */
    void *output;                 /* device pointer */
    int64_t output_stride;        /* samples */
    int32_t sample;               /* enum dsmvc_gb_sample */
    int32_t vectors;
    dsmvc_gb_conversion conversion;
} dsmvc_gb_plane_task;

typedef struct dsmvc_gb_executor dsmvc_gb_executor;
typedef double (*dsmvc_gb_custom_kernel)(double x, void *user);

/* ---- status --------------------------------------------------------- */
const char *dsmvc_gb_last_error(void);
int dsmvc_gb_abi_version(void);
/* Nonzero when a CUDA device is visible (dsmvc::cuda_available,
 * include/dsmvc/engine.hpp:204). */
int dsmvc_gb_cuda_available(void);

/* ---- planner (host, FP64) -------------------------------------------- */
/* build_axis_plan (include/dsmvc/engine.hpp:175-176,
 * src/axis_plan.cpp:1351).  `custom` is required for DSMVC_GB_CUSTOM. */
int dsmvc_gb_plan_build(const dsmvc_gb_axis_request *request,
                        dsmvc_gb_custom_kernel custom, void *user,
                        dsmvc_gb_plan **out);
/* get_or_build_axis_plan (engine.hpp:177-178, src/axis_plan.cpp:1358):
 * single-flight LRU shared by all callers; custom kernels are not cached. */
int dsmvc_gb_plan_get_or_build(const dsmvc_gb_axis_request *request,
                               dsmvc_gb_custom_kernel custom, void *user,
                               dsmvc_gb_plan **out);
void dsmvc_gb_plan_release(dsmvc_gb_plan *plan);
/* Builds `count` plans (no custom kernels) on up to `threads` host threads
 * (0 = one per hardware thread); the reference builds a sweep's plans one
 * Descale call at a time.  On failure no plan is returned and the message
 * names the first failing index. */
int dsmvc_gb_plan_build_many(const dsmvc_gb_axis_request *requests,
                             int32_t count, int32_t threads,
                             dsmvc_gb_plan **out);
/* The same plans with their numerical part computed on GPU `device` (-1:
 * the current device): the normal-matrix band, its banded LDL^T factor, the
 * three-stage condition estimate and Float64 routing, and the Float32 solve
 * arrays, for all plans at once (src/axis_plan.cpp:628-967 run per plan on
 * the host by the reference); the geometry, kernel weights and A^T CSR stay
 * on up to `threads` host threads.  The plans equal dsmvc_gb_plan_build's
 * bit for bit (same plan hashes).  Custom kernels are refused. */
int dsmvc_gb_plan_build_many_device(const dsmvc_gb_axis_request *requests,
                                    int32_t count, int32_t device, int32_t threads,
                                    dsmvc_gb_plan **out);
int dsmvc_gb_plan_get_info(const dsmvc_gb_plan *plan, dsmvc_gb_plan_info *out);
/* Read-only view of one plan array: 0 transpose_offsets (u32),
 * 1 transpose_indices (i32), 2 transpose_weights (f32), 3 lower_ld (f32),
 * 4 upper_l (f32), 5 inverse_diagonal (f32), 6 transpose_weights_f64,
 * 7 normal_bands_f64, 8 ldlt_bands_f64, 9 inverse_diagonal_f64 (f64). */
int dsmvc_gb_plan_get_array(const dsmvc_gb_plan *plan, int32_t which,
                            const void **data, uint64_t *count);
/* The arrays and scalars of a plan built elsewhere -- a reference
 * dsmvc::AxisPlan (include/dsmvc/engine.hpp:82-107) -- described by
 * pointers and element counts (each vector's data() and size()).  A pointer
 * may be NULL only when its count is 0; the four Float64 arrays are all
 * present (a plan that needs Float64) or all empty. */
typedef struct dsmvc_gb_plan_arrays {
    int32_t source_size;
    int32_t destination_size;
    int32_t support;
    int32_t half_bandwidth;
    double active_length;
    double shift;
    double normal_rcond;
    double normal_inf_norm;
    const uint32_t *transpose_offsets;     uint64_t transpose_offsets_count;
    const int32_t *transpose_indices;      uint64_t transpose_indices_count;
    const float *transpose_weights;        uint64_t transpose_weights_count;
    const float *lower_ld;                 uint64_t lower_ld_count;
    const float *upper_l;                  uint64_t upper_l_count;
    const float *inverse_diagonal;         uint64_t inverse_diagonal_count;
    const double *transpose_weights_f64;   uint64_t transpose_weights_f64_count;
    const double *normal_bands_f64;        uint64_t normal_bands_f64_count;
    const double *ldlt_bands_f64;          uint64_t ldlt_bands_f64_count;
    const double *inverse_diagonal_f64;    uint64_t inverse_diagonal_f64_count;
} dsmvc_gb_plan_arrays;
/* Imports a plan built by the reference planner, for the reference's
 * CudaExecutor::prepare(std::shared_ptr<const AxisPlan>) and the executor
 * calls that take `const AxisPlan &` (src/cuda/cuda_executor.hpp:26-52,
 * include/dsmvc/engine.hpp:389): the arrays are copied, checked like
 * AxisPlan::check_valid (src/axis_plan.cpp:1259-1341) and returned as a
 * plan handle the executor treats like one it built.  An invalid plan is
 * DSMVC_GB_INVALID_ARGUMENT.  An imported plan carries no request:
 * dsmvc_gb_plan_hashes then needs one. */
int dsmvc_gb_plan_import(const dsmvc_gb_plan_arrays *arrays, dsmvc_gb_plan **out);
/* FNV-1a plan hashes of tests/numerical_conformance.hpp:193-248. */
int dsmvc_gb_plan_hashes(const dsmvc_gb_plan *plan,
                         const dsmvc_gb_axis_request *request,
                         uint64_t *f32_hash, uint64_t *complete_hash);
/* Which kernel family a Float32 plan runs on, and the packed records of the
 * streaming kernels (no reference counterpart: the reference's equivalent
 * choice is solve_partition::choose, src/solve_partition.cpp:32-57).
 * `forward`/`backward` may be NULL to query the sizes only. */
typedef struct dsmvc_gb_stream_info {
    int32_t eligible;            /* streaming kernels usable */
    int32_t window;              /* dense gather window */
    int32_t forward_stride;      /* floats per forward record */
    int32_t backward_stride;     /* floats per backward record */
    int32_t ring_ok_u16;         /* 16-byte u16 row loads fit the ring */
    int32_t ring_ok_u8;          /* 16-byte u8 row loads fit the ring */
    int32_t chunk;               /* destinations per register chunk */
    int32_t ring;                /* source samples per thread ring */
    double backward_transfer;    /* carry influence after one chunk */
    char reason[96];             /* why not eligible */
    int32_t ring_ok_transposed;  /* the 2D passes' warp-wide block feed fits */
    int32_t exact;               /* two-pass transposing kernels admitted */
    int32_t segmentable;         /* 2D passes may split vectors into segments */
    double forward_transfer;     /* history influence after one chunk */
    int32_t group_union;         /* grouped records' union (12, 16), 0 if none */
    int32_t group_stride;        /* floats per group of four destinations */
    int32_t f64_eligible;        /* Float64 two-pass transposing kernels admitted */
    int32_t f64_segmentable;     /* ... and their segments */
    int32_t f64_margin;          /* segment margin in chunks (0: none) */
    double f64_margin_transfer;  /* influence left after that margin (4 if none) */
    int32_t exact_margin;        /* two-pass Float32 kernels' segment margin (0: none) */
    double exact_margin_transfer;/* influence left after that margin (4 if none) */
} dsmvc_gb_stream_info;
int dsmvc_gb_plan_stream_info(const dsmvc_gb_plan *plan,
                              dsmvc_gb_stream_info *info, float *forward,
                              uint64_t forward_capacity, float *backward,
                              uint64_t backward_capacity);
/* The grouped forward records of the 2D chunk-delayed kernels (one group
 * per four destinations, group_stride floats each, whole chunks); `count`
 * receives the floats needed, `out` may be NULL to query it. */
int dsmvc_gb_plan_stream_groups(const dsmvc_gb_plan *plan, float *out, uint64_t capacity, uint64_t *count);
/* planner_cache_stats / clear_planner_caches (engine.hpp:179-180). */
int dsmvc_gb_planner_cache_stats(dsmvc_gb_planner_stats *out);
void dsmvc_gb_clear_planner_caches(void);

/* ---- executor -------------------------------------------------------- */
/* CudaExecutor() (src/cuda/cuda_executor.hpp:15); device < 0 uses the
 * current device.  Fails with DSMVC_GB_UNAVAILABLE without a CUDA device:
 * an explicit CUDA backend never falls back (src/backend.cpp:53-58). */
int dsmvc_gb_executor_create(int32_t device, dsmvc_gb_executor **out);
void dsmvc_gb_executor_destroy(dsmvc_gb_executor *executor);
/* Executor::prepare / seal (engine.hpp:383-385). */
int dsmvc_gb_prepare(dsmvc_gb_executor *executor, const dsmvc_gb_plan *plan);
/* Many Executor::prepare calls at once (a sweep's thousands of plans): the
 * plans' device images are packed on host threads and uploaded in one
 * allocation with one copy. */
int dsmvc_gb_prepare_many(dsmvc_gb_executor *executor, const dsmvc_gb_plan *const *plans,
                          int32_t count);
int dsmvc_gb_seal(dsmvc_gb_executor *executor);
int dsmvc_gb_executor_get_stats(dsmvc_gb_executor *executor,
                                dsmvc_gb_executor_stats *out);

/* Synchronous host-frame calls: Executor::inverse_rows, inverse_columns,
 * inverse_2d, inverse_2d_u8, inverse_2d_u16 (engine.hpp:452-489,
 * src/cuda/cuda_executor.hpp:27-52). */
int dsmvc_gb_inverse_rows(dsmvc_gb_executor *executor,
                          const dsmvc_gb_plan *plan,
                          const float *input, int64_t input_stride,
                          float *output, int64_t output_stride,
                          int32_t rows);
int dsmvc_gb_inverse_columns(dsmvc_gb_executor *executor,
                             const dsmvc_gb_plan *plan,
                             const float *input, int64_t input_stride,
                             float *output, int64_t output_stride,
                             int32_t columns);
int dsmvc_gb_inverse_2d(dsmvc_gb_executor *executor,
                        const dsmvc_gb_plan *horizontal,
                        const dsmvc_gb_plan *vertical,
                        const float *input, int64_t input_stride,
                        float *output, int64_t output_stride);
int dsmvc_gb_inverse_2d_u8(dsmvc_gb_executor *executor,
                           const dsmvc_gb_plan *horizontal,
                           const dsmvc_gb_plan *vertical,
                           const uint8_t *input, int64_t input_stride,
                           uint8_t *output, int64_t output_stride,
                           const dsmvc_gb_conversion *conversion);
int dsmvc_gb_inverse_2d_u16(dsmvc_gb_executor *executor,
                            const dsmvc_gb_plan *horizontal,
                            const dsmvc_gb_plan *vertical,
                            const uint16_t *input, int64_t input_stride,
                            uint16_t *output, int64_t output_stride,
                            const dsmvc_gb_conversion *conversion);

/* One host-frame plane (a 2D descale of `input` into `output`, host
 * buffers, strides in samples); `conversion` is read for integer samples. */
typedef struct dsmvc_gb_host_plane {
    const dsmvc_gb_plan *horizontal;
    const dsmvc_gb_plan *vertical;
    const void *input;            /* host */
    int64_t input_stride;         /* samples */
    void *output;                 /* host */
    int64_t output_stride;        /* samples */
    int32_t sample;               /* enum dsmvc_gb_sample */
    dsmvc_gb_conversion conversion;
} dsmvc_gb_host_plane;
/* Synchronous host-frame call over many planes (frames x planes; no
 * reference counterpart beyond one inverse_2d call per plane): the planes
 * travel in groups of about DSMVC_GB_PIPELINE_MB (default 96) MiB of input
 * and output (uploads in order on one stream, kernels on four workspace
 * streams, downloads in order on another), so the upload of one group, the
 * kernels of the previous group and the download of the one before overlap.  Each
 * output equals the per-plane call's.  Host buffers should be pinned for the
 * copies to overlap.  Float64 non-finite data in any plane fails the call. */
int dsmvc_gb_inverse_2d_planes(dsmvc_gb_executor *executor,
                               const dsmvc_gb_host_plane *planes, int32_t count);

/* Device-resident batch (replaces the reference's per-plane exported-frame
 * calls, src/cuda/cuda_executor.hpp:60-76, and its launch layer,
 * src/cuda/cuda_launch.hpp:11-149): every task is enqueued on `stream`
 * (a cudaStream_t; NULL = the executor's own stream).  With `synchronize`
 * nonzero the call waits and reports Float64 non-finite data; otherwise
 * dsmvc_gb_stream_check() does that after the work completes. */
int dsmvc_gb_run_batch(dsmvc_gb_executor *executor,
                       const dsmvc_gb_plane_task *tasks, int32_t count,
                       void *stream, int32_t synchronize);
int dsmvc_gb_stream_check(dsmvc_gb_executor *executor, void *stream);
/* Waits for `stream` and releases the executor's per-stream resources; call
 * it before destroying a stream that was passed to dsmvc_gb_run_batch. */
int dsmvc_gb_stream_release(dsmvc_gb_executor *executor, void *stream);

/* Prepared batch: the task list of dsmvc_gb_run_batch routed, packed and
 * uploaded once (job table, intermediate planes and a status word owned by
 * the batch), then launched any number of times.  No counterpart in the
 * reference, whose launch layer rebuilds its launch parameters for every
 * plane (src/cuda/cuda_launch.hpp:11-149).  dsmvc_gb_batch_launch issues
 * kernels only -- no copy, allocation or host synchronisation -- so it may
 * be captured into a CUDA graph; launches of one batch must be ordered (one
 * stream or a graph) because they share the batch's scratch.
 * dsmvc_gb_batch_check waits for `stream` and reports Float64 non-finite
 * data seen by any earlier launch.  The tasks' buffers, their plans and the
 * executor must outlive the batch. */
typedef struct dsmvc_gb_batch dsmvc_gb_batch;
int dsmvc_gb_batch_create(dsmvc_gb_executor *executor,
                          const dsmvc_gb_plane_task *tasks, int32_t count,
                          dsmvc_gb_batch **out);
int dsmvc_gb_batch_launch(dsmvc_gb_batch *batch, void *stream);
int dsmvc_gb_batch_check(dsmvc_gb_batch *batch, void *stream);
int dsmvc_gb_batch_info(const dsmvc_gb_batch *batch, int64_t *kernel_launches,
                        int64_t *scratch_bytes, int64_t *table_bytes);
/* A batch whose tasks run in `parts` parts: 1 as one sequence of kernels;
 * 2 split where the source pixels are halved, the halves launched on
 * `stream` and on a stream of the batch forked from it and joined back to it
 * (stream-ordered, capturable), so that one half's second pass overlaps the
 * other's first; 0 (what dsmvc_gb_batch_create does) chooses 2 for 8 tasks
 * or more.  dsmvc_gb_batch_parts reports the count. */
int dsmvc_gb_batch_create_parts(dsmvc_gb_executor *executor,
                                const dsmvc_gb_plane_task *tasks, int32_t count,
                                int32_t parts, dsmvc_gb_batch **out);
int dsmvc_gb_batch_parts(const dsmvc_gb_batch *batch, int32_t *parts);
void dsmvc_gb_batch_destroy(dsmvc_gb_batch *batch);

/* Allocation-free 2D descale.  No counterpart in the reference.  For callers
 * that cannot allocate device memory (code running inside another
 * framework's memory pool, allocator-free real-time pipelines): the Float32
 * route of the 2D descale on device pointers, enqueued on `stream` (a
 * cudaStream_t; NULL = the legacy default stream), with no cudaMalloc,
 * cudaFree or other allocating call.  Its scratch lives in one file-scope
 * device array of DSMVC_GB_NOALLOC_SCRATCH_BYTES that every GPU loading this
 * library holds until the process exits.  A frame needs, each part rounded
 * up to 256 bytes: the job table; both plans' coefficients; the Float32
 * intermediate plane, 4 x vertical source size x horizontal destination
 * size bytes; and, for u8 or u16 output only, a forward plane of 4 x
 * vertical destination size x horizontal destination size bytes.  Frames
 * that need more, and plans that need Float64, are rejected with
 * DSMVC_GB_INVALID_ARGUMENT.  The first call on a device looks the array up
 * (cudaGetSymbolAddress) and keeps the address for the life of the process:
 * do not call this on a device after cudaDeviceReset.  Every call copies the
 * job table and the plans' coefficients from pageable host memory, so it may
 * block the host until those copies are done, and it returns
 * DSMVC_GB_INVALID_ARGUMENT on a stream that is being captured.  All calls
 * share the array: calls whose work overlaps on the GPU race, so order them
 * on one stream.  `sample` is an enum dsmvc_gb_sample; `conversion` is read
 * for integer samples. */
#define DSMVC_GB_NOALLOC_SCRATCH_BYTES (32u << 20)
int dsmvc_gb_inverse_2d_noalloc(const dsmvc_gb_plan *horizontal,
                                const dsmvc_gb_plan *vertical, int32_t sample,
                                const void *input, int64_t input_stride,
                                void *output, int64_t output_stride,
                                const dsmvc_gb_conversion *conversion,
                                void *stream);

/* Batched candidate sweep (the reference's native-resolution scan, where
 * each candidate is a Descale call, a resize back to the source size and a
 * PlaneStats average, docs/release-benchmark.md "getfnative"): every
 * candidate (a horizontal and a vertical plan over the same source size) is
 * descaled from one device frame, re-upscaled with its plans' forward
 * operators and scored by the mean absolute error against the frame.  The
 * scoring runs in a kernel of its own over each descaled plane or, with
 * `fused_scoring`, inside each candidate's columns pass where the pass and
 * the operators allow it (the descaled plane never reaches HBM, the sweep
 * needs a fraction of the memory; `fused_candidates` counts them).  The
 * candidates run in waves within `memory_budget` bytes (0 = 32 GiB), one
 * prepared batch per wave, the whole sweep captured into one CUDA graph
 * (`graph`), with CTA sizes and the scoring row segment chosen by timing the
 * alternatives on the first wave (`autotune`).  dsmvc_gb_sweep_run enqueues
 * the sweep on `stream`; dsmvc_gb_sweep_run_plain runs the same candidates one
 * at a time, each waited for (the per-frame baseline); dsmvc_gb_sweep_scores
 * waits and copies `count` scores in candidate order.  The frame and the
 * plans must outlive the sweep (the sweep keeps its own plan references). */
typedef struct dsmvc_gb_sweep dsmvc_gb_sweep;
typedef struct dsmvc_gb_sweep_options {
    int64_t memory_budget;
    int32_t autotune;
    int32_t graph;
    int32_t fused_scoring;        /* 1: score inside the columns pass where possible */
    int32_t reserved;             /* 0 */
} dsmvc_gb_sweep_options;
typedef struct dsmvc_gb_sweep_info {
    int32_t candidates;
    int32_t waves;
    int64_t device_bytes;
    int64_t kernel_launches;      /* per dsmvc_gb_sweep_run */
    double tune_milliseconds;
    int32_t segment_rows;
    int32_t tuned_groups;
    int32_t vectors_per_warp;     /* right-hand sides per warp the tuning chose: 32 or 64 */
    int32_t fused_candidates;     /* scored inside their columns pass */
} dsmvc_gb_sweep_info;
int dsmvc_gb_sweep_create(dsmvc_gb_executor *executor,
                          const dsmvc_gb_plan *const *horizontal,
                          const dsmvc_gb_plan *const *vertical, int32_t count,
                          const float *frame, int64_t frame_stride,
                          const dsmvc_gb_sweep_options *options,
                          dsmvc_gb_sweep **out);
int dsmvc_gb_sweep_run(dsmvc_gb_sweep *sweep, void *stream);
int dsmvc_gb_sweep_run_plain(dsmvc_gb_sweep *sweep, void *stream);
int dsmvc_gb_sweep_scores(dsmvc_gb_sweep *sweep, float *scores, void *stream);
int dsmvc_gb_sweep_get_info(const dsmvc_gb_sweep *sweep, dsmvc_gb_sweep_info *out);
/* Runs the sweep once without its graph, timing its stages with CUDA
 * events; `milliseconds[3]` receives the descale passes, the re-upscale with
 * the error sums and the score reduction. */
int dsmvc_gb_sweep_profile(dsmvc_gb_sweep *sweep, void *stream, double *milliseconds);
void dsmvc_gb_sweep_destroy(dsmvc_gb_sweep *sweep);

/* Host block registry: the reference's direct block registration for its
 * CUDA domain (include/dsmvc/host_blocks.hpp, src/host_blocks.cpp,
 * src/vs_frame_memory.cpp).  A frame host reports the host blocks (frame
 * pool allocations) its planes live in before each transfer; a block is
 * page-locked (cudaHostRegister) on its second use while the owner's
 * registered bytes stay within its limit (set_limit; 0, the default,
 * registers nothing), after which copies from and to planes inside it run
 * as DMA.  A block someone else page-locked counts as registered and is
 * never unregistered here.  Owners are opaque tokens.  release must come
 * before a block is freed; drop_owner releases all of an owner's blocks.
 * covered tells whether a range lies in a registered block.
 * dsmvc_gb_host_blocks_test_registrar replaces the CUDA calls (releasing
 * everything first) for tests: 0 CUDA, 1 a fake that registers, 2 a fake
 * that finds every block registered by someone else, 3 a fake that fails. */
typedef struct dsmvc_gb_host_block_stats {
    uint64_t registrations;       /* blocks registered (ours or foreign) */
    uint64_t failures;
    uint64_t cap_refusals;        /* second uses refused by the owner's limit */
    uint64_t hits;                /* covered() inside a registered block */
    uint64_t misses;
    uint64_t released;            /* blocks unregistered by the registry */
    uint64_t registered_bytes;    /* currently registered by the registry */
    uint64_t peak_bytes;
} dsmvc_gb_host_block_stats;
int dsmvc_gb_host_blocks_set_limit(const void *owner, int64_t bytes);
int dsmvc_gb_host_blocks_note_use(const void *owner, void *base, int64_t size);
int dsmvc_gb_host_blocks_covered(const void *pointer, int64_t bytes, int32_t *covered);
int dsmvc_gb_host_blocks_release(void *base, int64_t size);
int dsmvc_gb_host_blocks_drop_owner(const void *owner);
int dsmvc_gb_host_blocks_get_stats(dsmvc_gb_host_block_stats *out);
int dsmvc_gb_host_blocks_test_registrar(int32_t mode);

/* One block's page-locking, for a frame host that keeps its own registry
 * (the reference engine's, include/dsmvc/host_blocks.hpp): the CUDA
 * domain's Registrar of the reference's backend
 * (src/cuda/cuda_executor.cpp:1327-1361, installed at 1425-1441).
 * dsmvc_gb_host_register page-locks [base, base + size) for this library's
 * copies (cudaHostRegister, portable) and sets *outcome to 0 (page-locked
 * here: the caller unregisters it), 1 (already page-locked by someone
 * else: usable, never to be unregistered by the caller) or -1 (failed:
 * copies from and to it stay staged by the driver; the call still returns
 * DSMVC_GB_OK).  dsmvc_gb_host_unregister undoes an outcome of 0. */
int dsmvc_gb_host_register(void *base, int64_t size, int32_t *outcome);
int dsmvc_gb_host_unregister(void *base);

/* Request loop (continuous batching; no reference counterpart beyond its
 * synchronous per-frame calls on execution slots,
 * src/cuda/cuda_executor.cpp:1462-1503).  Requests of one or more 2D planes
 * (host buffers, any plans, sizes, kernels and precisions) are queued by
 * dsmvc_gb_server_submit and taken by `streams` worker threads, each forming
 * one batch of every queued request that fits the device arena of
 * `memory_budget` bytes (0 = 8 GiB), at most `max_batch` requests: uploads,
 * one executor batch, downloads.  Requests arriving while batches run join
 * the next batch as memory frees up, so the batches of the workers overlap
 * on the device.  Unprepared plans stay in the executor's device plan cache.
 * A request larger than the arena is refused (DSMVC_GB_LENGTH_ERROR).
 * dsmvc_gb_server_wait blocks until the request is done, returns its status
 * (its message through dsmvc_gb_last_error) and releases the ticket; host
 * buffers must stay valid until then.  A request's output does not depend on
 * the requests batched with it.  Latencies are measured from submission to
 * completion. */
typedef struct dsmvc_gb_server dsmvc_gb_server;
typedef struct dsmvc_gb_server_options {
    int64_t memory_budget;
    int32_t streams;      /* 1..16 */
    int32_t max_batch;    /* >= 1 */
} dsmvc_gb_server_options;
typedef struct dsmvc_gb_server_stats {
    uint64_t submitted;
    uint64_t completed;           /* including failed */
    uint64_t failed;
    uint64_t batches;
    double latency_p50_ms;
    double latency_p99_ms;
    double latency_mean_ms;
    double latency_max_ms;
    int64_t peak_device_bytes;
    uint64_t source_pixels;       /* of completed requests */
    double mean_batch_requests;
} dsmvc_gb_server_stats;
int dsmvc_gb_server_create(dsmvc_gb_executor *executor, const dsmvc_gb_server_options *options,
                           dsmvc_gb_server **out);
int dsmvc_gb_server_submit(dsmvc_gb_server *server, const dsmvc_gb_host_plane *planes,
                           int32_t count, uint64_t *ticket);
int dsmvc_gb_server_wait(dsmvc_gb_server *server, uint64_t ticket);
int dsmvc_gb_server_poll(dsmvc_gb_server *server, uint64_t ticket, int32_t *done);
int dsmvc_gb_server_get_stats(dsmvc_gb_server *server, dsmvc_gb_server_stats *out);
/* Clears the latency record and counters (not `submitted`). */
int dsmvc_gb_server_reset_stats(dsmvc_gb_server *server);
/* Finishes queued and running requests, then releases the server. */
void dsmvc_gb_server_destroy(dsmvc_gb_server *server);

/* Measured FP64 throughput of `device` in TFLOP/s (two per FMA), the
 * denominator of the Float64 route's FLOP roofline. */
int dsmvc_gb_measure_fp64_peak(int32_t device, double *tflops);

/* Kernel timing (the reference's NVTX ranges, src/cuda/nvtx.hpp:11-60, are
 * replaced by CUDA events): while enabled, every launch is bracketed by
 * events on its stream; dsmvc_gb_profile_read waits for them and returns one
 * entry per kernel name with its launch count, summed milliseconds and the
 * compulsory bytes (first-pass input + last-pass output) of those launches.
 * Enabling clears earlier records. */
typedef struct dsmvc_gb_kernel_time {
    char name[64];
    uint64_t launches;
    double milliseconds;
    uint64_t bytes;
} dsmvc_gb_kernel_time;
int dsmvc_gb_profile(dsmvc_gb_executor *executor, int32_t enable);
int dsmvc_gb_profile_read(dsmvc_gb_executor *executor,
                          dsmvc_gb_kernel_time *out, int32_t capacity,
                          int32_t *count);

#ifdef __cplusplus
}
#endif

#endif /* DSMVC_GB300_H */
