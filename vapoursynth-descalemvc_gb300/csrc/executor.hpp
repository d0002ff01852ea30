// GB300 descale executor: the backend behind the C ABI (capi.cpp).
//
// Mirrors the reference's CUDA executor contract (src/cuda/cuda_executor.hpp:
// 11-110, include/dsmvc/engine.hpp:363-504): plans are prepared once and
// sealed, host-frame calls are synchronous (the output is written when the
// call returns), strides are in samples, row padding is never read past the
// logical width nor written, and a Float64 plan on either axis sends the
// whole 2D call through the Float64 route, which raises on non-finite data.
// Added for GPU-resident callers: device-pointer calls enqueued on a stream
// and batched submissions of many planes (frames x planes, candidate sweeps)
// in one set of launches.
#pragma once

#include "kernels.cuh"
#include "planner.hpp"

#include <array>
#include <cstddef>
#include <cstdint>
#include <map>
#include <memory>
#include <string>
#include <vector>

namespace dsmvc_gb {

struct IntegerConversion {
    float input_offset = 0.0F;
    float input_scale = 1.0F;
    float output_scale = 1.0F;
    float output_offset = 0.0F;
    std::uint32_t output_maximum = 255U;
};

// One 2D plane of a batch, device pointers.  `horizontal` or `vertical` may
// be null for a one-axis descale of that plane (rows only / columns only).
struct PlaneTask {
    const AxisPlan *horizontal = nullptr;
    const AxisPlan *vertical = nullptr;
    const void *input = nullptr;
    std::ptrdiff_t input_stride = 0;    // samples
    void *output = nullptr;
    std::ptrdiff_t output_stride = 0;   // samples
    dev::Sample sample = dev::Sample::f32;
    IntegerConversion conversion{};
    // Source extent of a one-axis task: rows for rows-only, columns for
    // columns-only (ignored for 2D tasks).
    std::int32_t vectors = 0;
    // Optional owners of the plans.  A plan that was not prepared is looked
    // up in (or added to) the executor's device plan cache when its owner is
    // given; otherwise it is uploaded for this submission only.
    std::shared_ptr<const AxisPlan> horizontal_keep, vertical_keep;
    // Sweep scoring fused into the columns pass (Float32 2D tasks whose
    // vertical plan has an Executor::fused_scoring_window >= 0): a device
    // dev::ScoreEpilogue (score.cuh) and its tile count; `output` is then
    // not written (and may be null).
    const void *score = nullptr;
    std::int32_t score_tiles = 0;
};

// One host-frame plane of a multi-plane call (Executor::inverse_2d_planes).
struct HostPlane {
    const AxisPlan *horizontal = nullptr;
    const AxisPlan *vertical = nullptr;
    std::shared_ptr<const AxisPlan> horizontal_keep, vertical_keep;   // optional owners
    dev::Sample sample = dev::Sample::f32;
    const void *input = nullptr;        // host
    std::ptrdiff_t input_stride = 0;    // samples
    void *output = nullptr;             // host
    std::ptrdiff_t output_stride = 0;   // samples
    IntegerConversion conversion{};
};

// Per-kernel CUDA-event timing aggregated by kernel name; `bytes` counts the
// compulsory traffic of the launches (first-pass input, last-pass output).
struct KernelTime {
    std::string name;
    std::uint64_t launches = 0;
    double milliseconds = 0.0;
    std::uint64_t bytes = 0;
};

struct ExecutorStats {
    std::uint64_t launches = 0;        // kernel launches issued
    std::uint64_t plane_tasks = 0;
    std::uint64_t plan_uploads = 0;
    std::size_t device_plan_bytes = 0;
    std::size_t workspace_bytes = 0;
    // Device plan cache of plans that were not prepared (an LRU keyed by
    // plan identity and bounded by DSMVC_GB_PLAN_CACHE_MB, 16..4096 MiB,
    // default 2048: evicting frees device memory, which waits for the whole
    // device; the counterpart of DSMVC_CUDA_PLAN_CACHE_MB).
    std::uint64_t plan_cache_hits = 0;
    std::uint64_t plan_cache_misses = 0;
    std::uint64_t plan_cache_evictions = 0;
    std::size_t plan_cache_bytes = 0;
    // Host calls that repeated their slot's last task list and reused its
    // compiled launches (no routing, no plan lookups).
    std::uint64_t compile_reuses = 0;
};

class Executor;

// One launch group of a batch: every job of the group runs in one kernel
// launch.  `key` identifies the kernel variant (pass, kind, half-bandwidth,
// input and output sample kinds, window variant); `kind` 0/1 are the
// sequential Float32/Float64 kernels, 2 the streaming 1D kernels, 3 the
// transposing streaming 2D kernels.
struct BatchGroup {
    std::array<int, 6> key{};
    int kind = 0;
    int threads = 0;      // CTA size
    int blocks = 0;
    int jobs = 0;
    std::string name;
};

// CTA sizes chosen per launch-group key (an autotuner's output); groups not
// listed keep their kernel's default.  Kinds 0/1 accept 32..128, kind 3
// 32..256 (multiples of 32); kind 2 has a fixed size.
using BatchTuning = std::map<std::array<int, 6>, int>;

// A batch routed and packed once, with its own job table, scratch and status
// word on the device, then launched any number of times.  launch() issues
// kernels only (no copies, no allocation, no host synchronisation), so it
// can be captured into a CUDA graph.  The tasks' buffers and plans, and the
// executor, must outlive the batch.
class PreparedBatch {
public:
    struct Impl;
    explicit PreparedBatch(std::unique_ptr<Impl> impl);
    ~PreparedBatch();
    PreparedBatch(const PreparedBatch &) = delete;
    PreparedBatch &operator=(const PreparedBatch &) = delete;

    void launch(void *stream);
    // Launches group `index` alone (for timing one group).
    void launch_group(std::size_t index, void *stream);
    [[nodiscard]] std::vector<BatchGroup> groups() const;
    // Waits for `stream` and raises on a Float64 non-finite status (clears it).
    void check_status(void *stream);
    [[nodiscard]] std::size_t kernel_launches() const;
    [[nodiscard]] std::size_t scratch_bytes() const;
    [[nodiscard]] std::size_t table_bytes() const;
    // 1, or 2 when the tasks run as two overlapping parts.
    [[nodiscard]] std::size_t parts() const;

private:
    std::unique_ptr<Impl> impl_;
};

class Executor {
public:
    explicit Executor(int device = -1);
    ~Executor();
    Executor(const Executor &) = delete;
    Executor &operator=(const Executor &) = delete;

    [[nodiscard]] int device() const noexcept;

    // Uploads the plan's coefficients once; later calls with the same plan
    // object reuse them (keyed by identity, kept alive by the executor).
    void prepare(std::shared_ptr<const AxisPlan> plan);
    // Prepares many plans at once: their device images are packed on host
    // threads and uploaded in one allocation with one copy.
    void prepare_many(const std::vector<std::shared_ptr<const AxisPlan>> &plans);
    void seal();

    // Synchronous host-frame calls (reference Executor contract).
    // The optional owners let unprepared plans use the device plan cache.
    void inverse_rows(const AxisPlan &plan, const float *input, std::ptrdiff_t input_stride,
                      float *output, std::ptrdiff_t output_stride, std::int32_t rows,
                      const std::shared_ptr<const AxisPlan> &keep = nullptr);
    void inverse_columns(const AxisPlan &plan, const float *input, std::ptrdiff_t input_stride,
                         float *output, std::ptrdiff_t output_stride, std::int32_t columns,
                         const std::shared_ptr<const AxisPlan> &keep = nullptr);
    void inverse_2d(const AxisPlan &h, const AxisPlan &v, dev::Sample sample,
                    const void *input, std::ptrdiff_t input_stride, void *output,
                    std::ptrdiff_t output_stride, const IntegerConversion &conversion,
                    const std::shared_ptr<const AxisPlan> &h_keep = nullptr,
                    const std::shared_ptr<const AxisPlan> &v_keep = nullptr);

    // Synchronous host-frame call over many planes (frames x planes): the
    // planes go in groups of about `group_bytes` of input and output
    // (0: DSMVC_GB_PIPELINE_MB, default 96 MiB): uploads in order on one
    // stream, each group's kernels on one of four workspace streams,
    // downloads in order on another stream, so the upload of one group, the
    // kernels of the previous one and the download of the one before
    // overlap.  Results equal per-plane inverse_2d calls.
    // Host buffers should be pinned for the copies to overlap.
    void inverse_2d_planes(const std::vector<HostPlane> &planes, std::size_t group_bytes = 0);

    // Device-pointer batch: every task is enqueued on `stream` (null: the
    // executor's own).  With `synchronize` the call waits and raises on a
    // Float64 non-finite status; otherwise check_status() does that later.
    // With `scratch`, the intermediate planes live in that caller-owned
    // device buffer of `scratch_capacity` bytes instead of the stream's own.
    void run_batch(const std::vector<PlaneTask> &tasks, void *stream, bool synchronize,
                   void *scratch = nullptr, std::size_t scratch_capacity = 0);
    void check_status(void *stream);
    // Waits for `stream` and drops the executor's resources for it (call
    // before destroying a stream used with run_batch).
    void release_stream(void *stream);
    // Validates, routes and uploads `tasks` once (see PreparedBatch).  With
    // `scratch` the batch's intermediate planes live in that caller-owned
    // device buffer of `scratch_capacity` bytes (batches launched one after
    // another may share it); otherwise the batch allocates its own.
    // `vectors_per_warp` picks the transposing Float32 kernels' right-hand
    // sides per warp: 32 (one vector a lane), 64 (two a lane, the paired
    // kernels, where a plan admits them; same results bit for bit), or 0
    // for the executor's default (DSMVC_GB_PAIRED).  `parts`: 1 launches
    // every task in one sequence of kernels; 2 splits the tasks where the
    // source pixels are halved and launches the halves on the caller's
    // stream and a second one forked from it and joined back, so that one
    // half's second pass overlaps the other's first (measured 14 % faster on
    // 32 4K planes); 0 chooses 2 for batches of 8 tasks or more that own
    // their scratch.  Results do not depend on the parts beyond what
    // segment splits already allow (DSMVC_GB_SEGMENTS=1: none).
    [[nodiscard]] std::unique_ptr<PreparedBatch> prepare_batch(const std::vector<PlaneTask> &tasks,
                                                             const BatchTuning *tuning = nullptr,
                                                             void *scratch = nullptr,
                                                             std::size_t scratch_capacity = 0,
                                                             int vectors_per_warp = 0, int parts = 0);
    // Upper bound of the scratch bytes prepare_batch needs for `tasks`.
    [[nodiscard]] static std::size_t batch_scratch_bound(const std::vector<PlaneTask> &tasks);

    // The records window (0 for the plan's own, 8, 12 or 16) of the fused
    // scoring columns pass (PlaneTask::score) for Float32 2D tasks with this
    // vertical plan, or -1 where the plan's columns pass runs another kernel
    // (not chunk-delayed, half-bandwidth above 7, or DSMVC_GB_EXACT=1).  The
    // plan is uploaded (cached with its owner) as a batch would.
    [[nodiscard]] int fused_scoring_window(const AxisPlan &vertical,
                                           const std::shared_ptr<const AxisPlan> &keep = nullptr);

    [[nodiscard]] ExecutorStats stats() const;

    // Records CUDA events around every launch while enabled (enabling
    // clears earlier records); kernel_times() waits for them.
    void set_profiling(bool enable);
    [[nodiscard]] std::vector<KernelTime> kernel_times();

    struct Impl;

private:
    std::unique_ptr<Impl> impl_;
};

} // namespace dsmvc_gb
