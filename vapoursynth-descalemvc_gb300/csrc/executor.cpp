// GB300 descale executor (see executor.hpp).
//
// Device layout of one prepared plan: a single allocation holding the A^T CSR
// (offsets, indices, Float32 weights), the Float32 factor bands lower/upper,
// the inverse diagonal and, for plans that retain Float64, the Float64
// weights and LDL^T bands; every sub-array starts on a 256-byte boundary.
//
// A 2D plane runs as two batched launches per half-bandwidth group: the
// horizontal pass (one vector per source row) into a Float32 intermediate
// (Float64 in the Float64 route), then the vertical pass (one vector per
// destination column) into the output, with integer conversion fused into
// the load of the first pass and the store of the second.
#include "executor.hpp"
#include "copy.hpp"
#include "score.cuh"
#include "stream.cuh"
#include "stream_plan.hpp"

#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <list>
#include <map>
#include <mutex>
#include <stdexcept>
#include <string>
#include <tuple>
#include <cstdlib>
#include <functional>
#include <unordered_map>
#include <atomic>
#include <thread>
#include <vector>

namespace dsmvc_gb {
namespace {

void cuda_check(cudaError_t e, const char *what) {
    if (e != cudaSuccess)
        throw std::runtime_error(std::string("CUDA ") + what + ": " + cudaGetErrorString(e));
}
void cuda_check(int e, const char *what) { cuda_check(static_cast<cudaError_t>(e), what); }

constexpr std::size_t kAlign = 256;
constexpr int kSeqThreads = 128;   // threads per block of the sequential kernels
// Prepared batches of at least this many tasks (and their own scratch) run
// as two parts on two streams.
constexpr std::size_t kSplitBatchTasks = 8;
std::size_t align_up(std::size_t v) { return (v + kAlign - 1) / kAlign * kAlign; }

std::size_t sample_bytes(dev::Sample s) {
    switch (s) {
    case dev::Sample::u8: return 1;
    case dev::Sample::u16: return 2;
    case dev::Sample::f64: return 8;
    default: return 4;
    }
}

class DeviceBuffer {
public:
    DeviceBuffer() = default;
    DeviceBuffer(const DeviceBuffer &) = delete;
    DeviceBuffer &operator=(const DeviceBuffer &) = delete;
    ~DeviceBuffer() { release(); }
    void reserve(std::size_t bytes) {
        if (bytes <= bytes_) return;
        release();
        cuda_check(cudaMalloc(&ptr_, bytes), "allocating workspace");
        bytes_ = bytes;
    }
    void release() {
        if (ptr_) cudaFree(ptr_);
        ptr_ = nullptr;
        bytes_ = 0;
    }
    [[nodiscard]] char *data() const { return static_cast<char *>(ptr_); }
    [[nodiscard]] std::size_t size() const { return bytes_; }

private:
    void *ptr_ = nullptr;
    std::size_t bytes_ = 0;
};

struct DevicePlan {
    std::shared_ptr<const AxisPlan> keep;
    DeviceBuffer memory;
    // Plans prepared together share one allocation (upload_plans).
    std::shared_ptr<DeviceBuffer> arena;
    dev::PlanView view{};
    // Streaming-kernel records (when the plan qualifies, stream_plan.hpp).
    bool stream = false;
    bool stream_u16 = false, stream_u8 = false;
    bool stream_t = false;          // transposing 2D kernels admitted
    bool stream_x = false;          // two-pass transposing 2D kernels admitted
    bool stream_xg = false;         // ... with the grouped refill of window 8
    bool stream64 = false;          // Float64 two-pass transposing kernels admitted
    bool stream64_seg = false;      // ... and their segments (StreamPack64::segmentable)
    int margin64 = 0;
    std::vector<int> chunk_first_block64;
    dev::StreamPlanView stream_view64{};
    dev::StreamPlanView stream_view{};
    // Grouped forward records of the chunk-delayed transposing kernels
    // (StreamPack::forward_groups), when the plan has them: their union.
    int stream_union = 0;
    dev::StreamPlanView stream_view_g{};
    bool stream_p = false;          // paired transposing 2D kernels admitted
    dev::StreamPlanView stream_view2{};
    // Chunk-delayed transposing passes may split vectors into segments
    // (stream_plan.hpp); the ring's first block of each chunk.
    bool stream_seg = false;
    std::vector<int> chunk_first_block;
    // Two-pass transposing kernels in segments (StreamPack::exact_margin).
    int exact_margin = 0;
    std::size_t bytes = 0;
};

// Host image of a device plan: every array the kernels read, packed at
// 256-byte offsets, with the stream-kernel admission of the plan.
struct PlanImage {
    std::vector<char> bytes;
    std::vector<std::size_t> offsets;
    StreamPack pack;
    StreamPack64 pack64;
    std::size_t at_records = 0, at_paired = 0, at_records64 = 0, at_groups = 0;
};

PlanImage plan_image(const AxisPlan &p) {
    if (!p.valid()) throw std::invalid_argument("cannot prepare an invalid axis plan");
    const bool f64 = p.requires_float64();
    std::vector<std::pair<const void *, std::size_t>> parts = {
        {p.transpose_offsets.data(), p.transpose_offsets.size() * 4},
        {p.transpose_indices.data(), p.transpose_indices.size() * 4},
        {p.transpose_weights.data(), p.transpose_weights.size() * 4},
        {p.lower_ld.data(), p.lower_ld.size() * 4},
        {p.upper_l.data(), p.upper_l.size() * 4},
        {p.inverse_diagonal.data(), p.inverse_diagonal.size() * 4},
        {f64 ? p.transpose_weights_f64.data() : nullptr, f64 ? p.transpose_weights_f64.size() * 8 : 0},
        {f64 ? p.ldlt_bands_f64.data() : nullptr, f64 ? p.ldlt_bands_f64.size() * 8 : 0},
        {f64 ? p.normal_bands_f64.data() : nullptr, f64 ? p.normal_bands_f64.size() * 8 : 0},
    };
    PlanImage img;
    img.pack = pack_stream_plan(p, kStreamChunk, kStreamRing, stream_supports(p.half_bandwidth),
                                tsolve_supports(p.half_bandwidth));
    img.pack64 = pack_stream_plan64(p, kStreamChunk, kStreamRing, tsolve_supports(p.half_bandwidth));
    const StreamPack &pack = img.pack;
    const StreamPack64 &pack64 = img.pack64;
    std::size_t &at_records = img.at_records, &at_paired = img.at_paired, &at_records64 = img.at_records64,
                &at_groups = img.at_groups;
    if (pack.eligible || pack.exact) {
        at_records = parts.size();
        parts.push_back({pack.forward.data(), pack.forward.size() * 4});
        parts.push_back({pack.backward.data(), pack.backward.size() * 4});
        if (pack.group_union) {
            at_groups = parts.size();
            parts.push_back({pack.forward_groups.data(), pack.forward_groups.size() * 4});
            parts.push_back({pack.backward_groups.data(), pack.backward_groups.size() * 4});
        }
        if (pack.paired) {
            at_paired = parts.size();
            parts.push_back({pack.paired_forward.data(), pack.paired_forward.size() * 4});
            parts.push_back({pack.paired_backward.data(), pack.paired_backward.size() * 4});
        }
    }
    if (pack64.eligible) {
        at_records64 = parts.size();
        parts.push_back({pack64.forward.data(), pack64.forward.size() * 8});
        parts.push_back({pack64.backward.data(), pack64.backward.size() * 8});
    }
    std::size_t total = 0;
    for (auto &part : parts) {
        img.offsets.push_back(total);
        total += align_up(std::max<std::size_t>(part.second, 1));
    }
    img.bytes.assign(total, 0);
    for (std::size_t i = 0; i < parts.size(); ++i)
        if (parts[i].second) std::memcpy(img.bytes.data() + img.offsets[i], parts[i].first, parts[i].second);
    return img;
}

// Fills a device plan's views for its image uploaded at `base`.
void finish_plan(DevicePlan *dp, const AxisPlan &p, const PlanImage &img, char *base) {
    const bool f64 = p.requires_float64();
    const StreamPack &pack = img.pack;
    const StreamPack64 &pack64 = img.pack64;
    const std::vector<std::size_t> &offsets = img.offsets;
    const std::size_t at_records = img.at_records, at_paired = img.at_paired, at_records64 = img.at_records64,
                      at_groups = img.at_groups;
    const std::size_t total = img.bytes.size();
    auto &v = dp->view;
    v.source_size = p.source_size;
    v.destination_size = p.destination_size;
    v.half_bandwidth = p.half_bandwidth;
    v.retains_f64 = f64 ? 1 : 0;
    v.offsets = reinterpret_cast<const std::uint32_t *>(base + offsets[0]);
    v.indices = reinterpret_cast<const std::int32_t *>(base + offsets[1]);
    v.weights = reinterpret_cast<const float *>(base + offsets[2]);
    v.lower = reinterpret_cast<const float *>(base + offsets[3]);
    v.upper = reinterpret_cast<const float *>(base + offsets[4]);
    v.inv_diag = reinterpret_cast<const float *>(base + offsets[5]);
    v.weights64 = f64 ? reinterpret_cast<const double *>(base + offsets[6]) : nullptr;
    v.bands64 = f64 ? reinterpret_cast<const double *>(base + offsets[7]) : nullptr;
    v.normal64 = f64 ? reinterpret_cast<const double *>(base + offsets[8]) : nullptr;
    if (pack.eligible || pack.exact) {
        dp->stream = pack.eligible;
        dp->stream_u16 = pack.eligible && pack.ring_ok_u16;
        dp->stream_u8 = pack.eligible && pack.ring_ok_u8;
        dp->stream_t = pack.eligible && pack.ring_ok_transposed;
        dp->stream_seg = dp->stream_t && pack.segmentable;
        dp->exact_margin = pack.exact_margin;
        if (dp->stream_seg || dp->exact_margin) dp->chunk_first_block = pack.chunk_first_block;
        dp->stream_x = pack.exact;
        dp->stream_xg = pack.exact && pack.ring_ok_transposed && pack.window == 8;
        auto &sv = dp->stream_view;
        sv.source_size = p.source_size;
        sv.destination_size = p.destination_size;
        sv.half_bandwidth = p.half_bandwidth;
        sv.window = pack.window;
        sv.forward_stride = pack.forward_stride;
        sv.backward_stride = pack.backward_stride;
        sv.forward = reinterpret_cast<const float *>(base + offsets[at_records]);
        sv.backward = reinterpret_cast<const float *>(base + offsets[at_records + 1]);
        if (pack.group_union) {
            dp->stream_union = pack.group_union;
            dp->stream_view_g = sv;
            dp->stream_view_g.window = pack.group_union;
            dp->stream_view_g.forward_stride = pack.group_stride / 4;
            dp->stream_view_g.forward = reinterpret_cast<const float *>(base + offsets[at_groups]);
            dp->stream_view_g.backward_stride = (4 * p.half_bandwidth + 3) / 4;
            dp->stream_view_g.backward = reinterpret_cast<const float *>(base + offsets[at_groups + 1]);
        }
        if (pack.paired) {
            dp->stream_p = true;
            auto &pv = dp->stream_view2;
            pv = sv;
            pv.forward_stride = pack.paired_forward_stride;
            pv.backward_stride = pack.paired_backward_stride;
            pv.forward = reinterpret_cast<const float *>(base + offsets[at_paired]);
            pv.backward = reinterpret_cast<const float *>(base + offsets[at_paired + 1]);
        }
    }
    if (pack64.eligible) {
        dp->stream64 = true;
        dp->stream64_seg = pack64.segmentable;
        if (pack64.segmentable) {
            dp->margin64 = pack64.margin;
            dp->chunk_first_block64 = pack64.chunk_first_block;
        }
        auto &xv = dp->stream_view64;
        xv.source_size = p.source_size;
        xv.destination_size = p.destination_size;
        xv.half_bandwidth = p.half_bandwidth;
        xv.window = pack64.window;
        xv.forward_stride = pack64.forward_stride;
        xv.backward_stride = pack64.backward_stride;
        xv.forward = reinterpret_cast<const float *>(base + offsets[at_records64]);
        xv.backward = reinterpret_cast<const float *>(base + offsets[at_records64 + 1]);
    }
    dp->bytes = total;
}

std::shared_ptr<DevicePlan> upload_plan(const AxisPlan &p, std::shared_ptr<const AxisPlan> keep) {
    if (!p.valid()) throw std::invalid_argument("cannot prepare an invalid axis plan");
    const PlanImage img = plan_image(p);
    auto dp = std::make_shared<DevicePlan>();
    dp->memory.reserve(img.bytes.size());
    cuda_check(cudaMemcpy(dp->memory.data(), img.bytes.data(), img.bytes.size(), cudaMemcpyHostToDevice),
               "uploading plan");
    finish_plan(dp.get(), p, img, dp->memory.data());
    dp->keep = std::move(keep);
    return dp;
}

// Many plans: images packed on host threads, one device allocation shared by
// the plans (held until the last of them is released) and one copy.
std::vector<std::shared_ptr<DevicePlan>> upload_plans(const std::vector<std::shared_ptr<const AxisPlan>> &plans) {
    const std::size_t count = plans.size();
    std::vector<PlanImage> images(count);
    std::vector<std::string> errors(count);
    std::atomic<std::size_t> next{0};
    auto worker = [&] {
        for (std::size_t i = next++; i < count; i = next++) {
            try {
                if (!plans[i] || !plans[i]->valid()) throw std::invalid_argument("cannot prepare an invalid axis plan");
                images[i] = plan_image(*plans[i]);
            } catch (const std::exception &e) {
                errors[i] = e.what();
            }
        }
    };
    const unsigned n = std::max(1U, std::min<unsigned>(std::thread::hardware_concurrency(),
                                                       static_cast<unsigned>(std::max<std::size_t>(count, 1))));
    std::vector<std::thread> pool;
    for (unsigned t = 1; t < n; ++t) pool.emplace_back(worker);
    worker();
    for (auto &t : pool) t.join();
    for (const auto &e : errors)
        if (!e.empty()) throw std::invalid_argument(e);
    std::vector<std::size_t> at(count);
    std::size_t total = 0;
    for (std::size_t i = 0; i < count; ++i) {
        at[i] = total;
        total += align_up(std::max<std::size_t>(images[i].bytes.size(), 1));
    }
    std::vector<std::shared_ptr<DevicePlan>> out;
    if (count == 0) return out;
    auto arena = std::make_shared<DeviceBuffer>();
    arena->reserve(total);
    {
        std::vector<char> host(total, 0);
        for (std::size_t i = 0; i < count; ++i)
            std::memcpy(host.data() + at[i], images[i].bytes.data(), images[i].bytes.size());
        cuda_check(cudaMemcpy(arena->data(), host.data(), total, cudaMemcpyHostToDevice), "uploading plans");
    }
    out.reserve(count);
    for (std::size_t i = 0; i < count; ++i) {
        auto dp = std::make_shared<DevicePlan>();
        finish_plan(dp.get(), *plans[i], images[i], arena->data() + at[i]);
        dp->arena = arena;
        dp->keep = plans[i];
        out.push_back(std::move(dp));
    }
    return out;
}

// Per-stream scratch: intermediate, forward scratch, staged host frames, job
// table and the Float64 status word.
struct Workspace {
    cudaStream_t stream = nullptr;
    bool owns_stream = false;
    DeviceBuffer scratch;
    DeviceBuffer staging;
    DeviceBuffer jobs;
    // The status word in mapped page-locked memory: kernels set bits through
    // `status` (its device address), the host reads `status_host` once the
    // stream is done, with no copy.
    std::uint32_t *status = nullptr;
    std::uint32_t *status_host = nullptr;
    // A kernel that may set the status word ran on this stream since the
    // status was last read.
    bool status_pending = false;
    // The last few compiled task lists (Executor::Impl::Compiled,
    // type-erased), most recent first, reused when a call repeats one (same
    // plans with their owners, pointers, strides, conversion) and the
    // scratch has not moved: a frame server alternates the luma and chroma
    // planes of its frames through one slot.
    // Each entry keeps its job table on the device, copied once: a repeated
    // call launches with no copy.
    struct CompiledEntry {
        std::shared_ptr<void> compiled;
        std::vector<PlaneTask> tasks;
        char *scratch = nullptr;
        std::unique_ptr<DeviceBuffer> table;
    };
    static constexpr std::size_t kCompiledEntries = 4;
    std::vector<CompiledEntry> compiled;
    std::vector<char> host_table;
    // Job tables travel through two pinned slots, each reused only after
    // its previous copy has finished; an unchanged table is not copied.
    char *pinned[2] = {nullptr, nullptr};
    std::size_t pinned_bytes[2] = {0, 0};
    cudaEvent_t pinned_done[2] = {nullptr, nullptr};
    int pinned_next = 0;
    std::vector<char> device_table;   // what ws.jobs holds

    // Copies `table` into `dst` through a pinned slot, on `copies` (the
    // workspace's own stream by default; the caller then orders the kernels
    // after it).  No kernel still to run may read `dst`'s old contents: on
    // the workspace's stream the copy follows them, and a caller passing a
    // copy stream has made it wait for them.
    void copy_table(DeviceBuffer &dst, const std::vector<char> &table, cudaStream_t copies) {
        const cudaStream_t s = copies ? copies : stream;
        dst.reserve(table.size());
        const int k = pinned_next;
        pinned_next ^= 1;
        if (pinned_done[k]) cuda_check(cudaEventSynchronize(pinned_done[k]), "waiting for a job table slot");
        else cuda_check(cudaEventCreateWithFlags(&pinned_done[k], cudaEventDisableTiming), "creating event");
        if (pinned_bytes[k] < table.size()) {
            if (pinned[k]) cudaFreeHost(pinned[k]);
            pinned[k] = nullptr;
            cuda_check(cudaMallocHost(&pinned[k], table.size()), "allocating a pinned job table");
            pinned_bytes[k] = table.size();
        }
        std::memcpy(pinned[k], table.data(), table.size());
        cuda_check(cudaMemcpyAsync(dst.data(), pinned[k], table.size(), cudaMemcpyHostToDevice, s),
                   "uploading job table");
        cuda_check(cudaEventRecord(pinned_done[k], s), "recording event");
    }
    // The shared job table `jobs` for task lists not kept in `compiled`.
    void upload_table(const std::vector<char> &table, cudaStream_t copies = nullptr) {
        if (table == device_table) return;
        copy_table(jobs, table, copies);
        device_table = table;
    }

    // The workspace's stream waits for the work issued so far on `copies`.
    cudaEvent_t copies_done = nullptr;
    void follow(cudaStream_t copies) {
        if (!copies_done) cuda_check(cudaEventCreateWithFlags(&copies_done, cudaEventDisableTiming), "creating event");
        cuda_check(cudaEventRecord(copies_done, copies), "recording event");
        cuda_check(cudaStreamWaitEvent(stream, copies_done, 0), "ordering kernels");
    }

    explicit Workspace(cudaStream_t s) : stream(s) {
        if (!stream) {
            cuda_check(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "creating stream");
            owns_stream = true;
        }
        cuda_check(cudaHostAlloc(reinterpret_cast<void **>(&status_host), sizeof(std::uint32_t), cudaHostAllocMapped),
                   "allocating status");
        *status_host = 0;
        cuda_check(cudaHostGetDevicePointer(reinterpret_cast<void **>(&status), status_host, 0), "mapping status");
    }
    ~Workspace() {
        // A caller's stream may already be destroyed: wait on what this
        // workspace owns (its own stream, its table copies) and let the
        // frees below wait for the device.
        if (owns_stream) cudaStreamSynchronize(stream);
        for (int k = 0; k < 2; ++k)
            if (pinned_done[k]) cudaEventSynchronize(pinned_done[k]);
        for (int k = 0; k < 2; ++k) {
            if (pinned[k]) cudaFreeHost(pinned[k]);
            if (pinned_done[k]) cudaEventDestroy(pinned_done[k]);
        }
        if (status_host) cudaFreeHost(status_host);
        if (copies_done) cudaEventDestroy(copies_done);
        if (owns_stream) cudaStreamDestroy(stream);
    }
};

// Workspaces of the multi-plane host call: a group's upload waits for the
// downloads of the group kPipeDepth before it (three left the last group of
// 64 YUV420P16 frames waiting 0.1 ms for one).
constexpr std::size_t kPipeDepth = 4;

// The multi-plane host call's copy streams: every upload in issue order on
// one stream, every download on another, linked to the workspaces' kernels
// by events (one set per workspace).  Copies issued on the workspaces' own
// streams ran concurrently, shared the link and finished out of order, so
// each group's kernels started late (64 YUV420P16 frames 1080p -> 810p:
// 2.45 ms a call, the last group waiting 0.11 ms for its workspace).
struct CopyLanes {
    cudaStream_t up = nullptr, down = nullptr;
    std::array<cudaEvent_t, kPipeDepth> computed{}, downloaded{};

    void create() {
        for (cudaStream_t *s : {&up, &down})
            if (!*s) cuda_check(cudaStreamCreateWithFlags(s, cudaStreamNonBlocking), "creating stream");
        for (auto *set : {&computed, &downloaded})
            for (auto &e : *set)
                if (!e) cuda_check(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "creating event");
    }
    void synchronize() const {
        for (cudaStream_t s : {up, down})
            if (s) cudaStreamSynchronize(s);
    }
    ~CopyLanes() {
        synchronize();
        for (auto *set : {&computed, &downloaded})
            for (auto e : *set)
                if (e) cudaEventDestroy(e);
        for (cudaStream_t s : {up, down})
            if (s) cudaStreamDestroy(s);
    }
};

struct DeviceGuard {
    int previous = -1;
    explicit DeviceGuard(int device) {
        cudaGetDevice(&previous);
        if (previous != device) cuda_check(cudaSetDevice(device), "selecting device");
    }
    ~DeviceGuard() {
        int now = -1;
        cudaGetDevice(&now);
        if (previous >= 0 && now != previous) cudaSetDevice(previous);
    }
};

} // namespace

struct Executor::Impl {
    int device = 0;
    mutable std::mutex mutex;
    std::unordered_map<const AxisPlan *, std::shared_ptr<DevicePlan>> plans;
    // Device plan cache of unprepared plans given with their owners: entries
    // hold the owner, so a key never outlives its plan; an evicted entry's
    // memory is released when the last submission holding it is done with it.
    struct CacheEntry {
        std::shared_ptr<DevicePlan> plan;
        std::list<const AxisPlan *>::iterator lru;
    };
    std::unordered_map<const AxisPlan *, CacheEntry> cache;
    std::list<const AxisPlan *> cache_lru;
    std::size_t cache_bytes = 0;
    std::size_t cache_capacity = 2048ULL << 20;
    bool sealed = false;
    // Synchronous host calls take one of these slots (the reference's
    // execution slots, src/cuda/cuda_executor.cpp:1102-1160).
    std::vector<std::unique_ptr<Workspace>> slots;
    std::vector<bool> slot_busy;
    // At most this many host calls run at once, each on its own stream
    // (DSMVC_GB_STREAMS=1..16, the counterpart of DSMVC_CUDA_STREAMS,
    // src/cuda/cuda_executor.cpp:105-118).  A single plane fills only a few
    // SMs, so concurrent calls are what keeps the GPU busy.
    std::size_t max_slots = 16;
    std::condition_variable slot_free;
    std::map<cudaStream_t, std::unique_ptr<Workspace>> stream_spaces;
    ExecutorStats stats;
    // Multi-plane host calls: kPipeDepth workspaces whose kernels run on
    // their own streams, the copies on two shared ones; one such call at a
    // time.
    std::mutex pipe_mutex;
    std::array<std::unique_ptr<Workspace>, kPipeDepth> pipe;
    CopyLanes pipe_copies;   // destroyed first: its streams wait for their copies
    std::size_t pipe_group_bytes = 96ULL << 20;
    // DSMVC_GB_HOST_DIRECT=1: planes of the multi-plane host call whose
    // buffers are page-locked host memory are read and written by the
    // kernels in place (mapped through unified addressing) instead of being
    // staged by copies.
    bool host_direct = false;
    // DSMVC_GB_FEED_STALL_TEST=1: the staged feeds wait for a barrier phase
    // nothing completes (tests of the bounded wait and its status report).
    bool feed_stall_test = false;

    // Optional per-launch CUDA-event timing (dsmvc_gb_profile).
    struct Record {
        std::string name;
        cudaEvent_t start = nullptr, stop = nullptr;
        std::uint64_t bytes = 0;
    };
    bool profiling = false;
    std::vector<cudaEvent_t> event_pool;   // reused across profiling sessions
    std::size_t events_used = 0;

    // Caller holds `mutex`.
    cudaEvent_t pooled_event() {
        if (events_used == event_pool.size()) {
            cudaEvent_t e = nullptr;
            cuda_check(cudaEventCreate(&e), "creating event");
            event_pool.push_back(e);
        }
        return event_pool[events_used++];
    }
    // DSMVC_GB_STREAM=0 keeps every plan on the sequential kernels (the
    // counterpart of the reference's DSMVC_GPU_SOLVE_PARTITION switch).
    bool allow_stream = true;
    // DSMVC_GB_PAIRED=1 runs admitted 2D planes on the paired transposing
    // kernels (64 vectors per warp); the unpaired ones (32 per warp) are the
    // default, faster on GB300 at the occupancy the paired ones reach.
    bool allow_paired = false;
    // DSMVC_GB_EXACT=1 runs every admitted 2D pass on the two-pass
    // transposing kernels; otherwise they serve the plans the chunk-delayed
    // kernels do not admit (slowly decaying factors, half-bandwidths 9, 11).
    bool prefer_exact = false;
    // The Float64 two-pass kernels fuse multiply-adds and multiply by the
    // reciprocal pivot (within the <= 1 float32 ULP contract, about half the
    // FP64 operations); DSMVC_GB_F64_EXACT=1 (or DSMVC_GB_EXACT=1) runs the
    // CPU scalar route's operation order, equal to it bit for bit.
    bool f64_fused = true;
    // DSMVC_GB_F64_REFINE=1: Float64 2D planes on the two-pass Float64
    // kernels add one residual refinement step per pass (refine64.cu): the
    // columns pass then writes a Float64 plane, refined and converted last.
    bool f64_refine = false;
    // Default CTA size of the transposing kernels (DSMVC_GB_TSTREAM_THREADS,
    // 32..256 in multiples of 32); batches may tune it per launch group.
    int tstream_threads = kTStreamThreads;
    // Segments of the chunk-delayed transposing passes (DSMVC_GB_SEGMENTS):
    // 0 automatic (a launch group whose warps leave the GPU's resident warp
    // slots unfilled splits its vectors into up to slots / warps ranges of
    // at least kMinSegmentChunks chunks), 1 never, N >= 2 exactly N per job
    // where admitted and long enough.
    int segment_mode = 0;
    int warp_slots = 0;      // SMs x resident warps of the transposing kernels
    std::vector<Record> records;

    // Prepared plans first, then the cache (plans with owners), else a
    // private upload for this submission (`held` keeps every non-prepared
    // device plan alive; `private_uploads` counts the uncached ones).
    const DevicePlan &device_plan(const AxisPlan &plan, const std::shared_ptr<const AxisPlan> &keep,
                                  std::vector<std::shared_ptr<DevicePlan>> &held, int &private_uploads) {
        {
            std::scoped_lock lock(mutex);
            if (auto it = plans.find(&plan); it != plans.end()) return *it->second;
            if (keep && keep.get() == &plan) {
                if (auto it = cache.find(&plan); it != cache.end()) {
                    cache_lru.splice(cache_lru.end(), cache_lru, it->second.lru);
                    ++stats.plan_cache_hits;
                    held.push_back(it->second.plan);
                    return *held.back();
                }
            }
        }
        if (!keep || keep.get() != &plan) {
            held.push_back(upload_plan(plan, nullptr));
            ++private_uploads;
            std::scoped_lock lock(mutex);
            ++stats.plan_uploads;
            return *held.back();
        }
        auto dp = upload_plan(plan, keep);
        std::scoped_lock lock(mutex);
        ++stats.plan_uploads;
        if (auto it = cache.find(&plan); it != cache.end()) {
            // Another thread uploaded it meanwhile.
            held.push_back(it->second.plan);
            return *held.back();
        }
        ++stats.plan_cache_misses;
        cache_lru.push_back(&plan);
        cache.emplace(&plan, CacheEntry{dp, std::prev(cache_lru.end())});
        cache_bytes += dp->bytes;
        while (cache_bytes > cache_capacity && cache.size() > 1) {
            const AxisPlan *victim = cache_lru.front();
            auto v = cache.find(victim);
            cache_bytes -= v->second.plan->bytes;
            cache_lru.pop_front();
            cache.erase(v);
            ++stats.plan_cache_evictions;
        }
        held.push_back(std::move(dp));
        return *held.back();
    }

    Workspace &acquire_slot(std::size_t &index) {
        std::unique_lock lock(mutex);
        for (;;) {
            for (std::size_t i = 0; i < slots.size(); ++i) {
                if (!slot_busy[i]) {
                    slot_busy[i] = true;
                    index = i;
                    return *slots[i];
                }
            }
            if (slots.size() < max_slots) {
                slots.push_back(std::make_unique<Workspace>(nullptr));
                slot_busy.push_back(true);
                index = slots.size() - 1;
                return *slots.back();
            }
            slot_free.wait(lock);
        }
    }

    void release_slot(std::size_t index) {
        {
            std::scoped_lock lock(mutex);
            slot_busy[index] = false;
        }
        slot_free.notify_one();
    }

    Workspace &stream_space(cudaStream_t stream) {
        std::scoped_lock lock(mutex);
        auto &ws = stream_spaces[stream];
        if (!ws) ws = std::make_unique<Workspace>(stream);
        return *ws;
    }

    // A routed, packed submission: launch groups over one job table.
    struct Launch {
        int pass, kind, hb;
        dev::Sample in, out;
        int variant;
        std::size_t offset;
        int count, blocks;
        std::uint64_t bytes;
        int record_floats;
        int threads;
    };
    // CTA size per launch group, keyed by (pass, kind, hb, in, out, variant);
    // groups not listed take the default size of their kernel.
    using GroupTuple = std::tuple<int, int, int, int, int, int>;
    using Tuning = std::map<GroupTuple, int>;
    struct Compiled {
        std::vector<std::shared_ptr<DevicePlan>> temporaries;   // non-prepared plans in use
        int private_uploads = 0;
        std::vector<char> table;
        std::vector<Launch> launches;
        std::size_t scratch_bytes = 0;
        std::size_t tasks = 0;
    };
    // Window of the fused scoring columns pass for this vertical plan, or -1.
    [[nodiscard]] int fused_window(const DevicePlan &dp) const;
    // `status`: the device status word the launches report to.
    void compile(const std::vector<PlaneTask> &tasks, Compiled &out,
                 const std::function<char *(std::size_t)> &scratch, std::uint32_t *status,
                 const Tuning *tuning = nullptr, int vectors_per_warp = 0);
    void launch(const Compiled &c, const char *device_table, cudaStream_t stream, std::uint32_t *status);
    // `copies`: a stream holding the tasks' input copies; the job table is
    // copied behind them there and the kernels wait for both.
    void enqueue(Workspace &ws, const std::vector<PlaneTask> &tasks, char *scratch = nullptr,
                 std::size_t scratch_capacity = 0, cudaStream_t copies = nullptr);
    void finish(Workspace &ws);
};

namespace {

// Launch groups: one launch per kernel variant, every job of a group shares
// half-bandwidth and sample kinds.
struct GroupKey {
    int pass;        // 0 first pass (rows), 1 second pass (columns)
    int kind;        // 0 sequential Float32, 1 sequential Float64, 2 streaming,
                     // 3 transposing streaming (2D), ... 9 columns pass with
                     // fused sweep scoring
    int hb;
    dev::Sample in, out;
    int variant = 0; // kind 3: the kernels' window (8, or 12 / 16 for grouped records), else 0
    bool operator<(const GroupKey &o) const {
        return std::tie(pass, kind, hb, in, out, variant)
            < std::tie(o.pass, o.kind, o.hb, o.in, o.out, o.variant);
    }
};

dev::Conversion to_dev(const IntegerConversion &c) {
    return {c.input_offset, c.input_scale, c.output_scale, c.output_offset, c.output_maximum};
}

bool stream_row_ok(const DevicePlan &dp, dev::Sample in) {
    if (!dp.stream) return false;
    if (in == dev::Sample::u16) return dp.stream_u16;
    if (in == dev::Sample::u8) return dp.stream_u8;
    return in == dev::Sample::f32;
}

// Launch-group variant of a transposing pass.  Chunk-delayed kernels: the
// union of grouped records (12, 16), else 8 for the window-8 kernels
// (compile-time gather), else 0.  Paired and two-pass kernels: 1 runs the
// window-8 kernels (for the two-pass ones also the grouped refill).
int compiled_window(const DevicePlan &dp, int kind) {
    if (kind == 5) return dp.stream_xg ? 1 : 0;
    if (kind == 3 && dp.stream_union) return dp.stream_union;
    return dp.stream_view.window == 8 ? (kind == 3 ? 8 : 1) : 0;
}

std::string kernel_name(const GroupKey &k);

} // namespace

int Executor::Impl::fused_window(const DevicePlan &dp) const {
    if (!allow_stream || prefer_exact || !dp.stream || !dp.stream_t) return -1;
    const int hb = dp.stream_view.half_bandwidth;
    if (hb < 1 || hb > 7) return -1;
    const int w = compiled_window(dp, 3);
    return w == 0 || w == 8 || w == 12 || w == 16 ? w : -1;
}

namespace {

std::string kernel_name(const GroupKey &k) {
    static const char *kinds[] = {"axis_f32", "axis_f64", "stream_f32", "tstream_f32", "tstream2_f32",
                                  "tsolve_f32", "tsolve_f64", "refine_f64", "convert_f64", "tscore_f32"};
    return std::string(kinds[k.kind]) + (k.pass ? "/columns" : "/rows") + "/hb" + std::to_string(k.hb);
}

} // namespace

namespace {

// Chunks of forward values the Float64 segments of one pass store: each
// segment's range with `margin` chunks on either side (within the vector).
std::size_t segment64_chunks(int destinations, int segments, int margin) {
    const int chunks = (destinations + kStreamChunk - 1) / kStreamChunk;
    std::size_t total = 0;
    for (int k = 0; k < segments; ++k) {
        const int begin = static_cast<int>(static_cast<long>(k) * chunks / segments);
        const int end = static_cast<int>(static_cast<long>(k + 1) * chunks / segments);
        total += static_cast<std::size_t>(std::min(end + margin, chunks) - std::max(begin - margin, 0));
    }
    return total;
}

// One two-pass job (Float64 or Float32), or its segments: chunk ranges with
// `margin` chunks on either side, each with its forward-value region in
// `yseg` (rows of `pitch` elements of `elem` bytes, starting at the
// segment's first computed chunk) and its ring's first block.
template <class Item>
void push_segments(std::vector<Item> &group, const Item &whole, const std::vector<int> &first_blocks, int margin,
                   int destinations, int segments, char *yseg, std::int64_t pitch, std::size_t elem) {
    if (segments <= 1) {
        group.push_back(whole);
        return;
    }
    const int chunks = (destinations + kStreamChunk - 1) / kStreamChunk;
    std::size_t at = 0;
    for (int k = 0; k < segments; ++k) {
        const int begin = static_cast<int>(static_cast<long>(k) * chunks / segments);
        const int end = static_cast<int>(static_cast<long>(k + 1) * chunks / segments);
        const int first = std::max(begin - margin, 0);
        const int last = std::min(end + margin, chunks);
        Item it = whole;
        it.stream.chunk_begin = begin;
        it.stream.chunk_end = end;
        it.stream.first_sample = first_blocks[static_cast<std::size_t>(first)];
        it.stream.margin = margin;
        it.stream.y = reinterpret_cast<float *>(yseg + at * kStreamChunk * static_cast<std::size_t>(pitch) * elem);
        it.stream.y_elem = pitch;
        at += static_cast<std::size_t>(last - first);
        group.push_back(it);
    }
}

// Jobs of a chunk-delayed transposing launch group (sorted by plan), split
// into segments of whole chunks.  Automatic mode: when the group's warps fill
// fewer than `slots` resident warp slots, up to slots / warps segments per
// job; each segment spans at least kMinSegmentChunks chunks, and only plans
// whose forward warm-up is admitted split.  Per plan, the jobs come segment
// by segment, so that only plan and segment changes round up to whole CTAs.
template <class Item>
std::vector<Item> segment_items(const std::vector<Item> &items, int vectors_per_warp, int mode, int slots) {
    if (mode == 1) return items;
    int segments = mode;
    if (mode == 0) {
        long warps = 0;
        for (const auto &it : items) warps += (it.stream.vectors + vectors_per_warp - 1) / vectors_per_warp;
        if (warps <= 0 || slots <= 0) return items;
        segments = static_cast<int>(std::min<long>(slots / warps, 64));
        if (segments < 2) return items;
    }
    std::vector<Item> out;
    out.reserve(items.size());
    for (std::size_t i = 0; i < items.size();) {
        std::size_t j = i;
        while (j < items.size() && items[j].stream.plan.forward == items[i].stream.plan.forward) ++j;
        const DevicePlan *dp = items[i].plan;
        const int chunks = (items[i].stream.plan.destination_size + kStreamChunk - 1) / kStreamChunk;
        const int s = dp && dp->stream_seg ? std::max(1, std::min(segments, chunks / kMinSegmentChunks)) : 1;
        for (int k = 0; k < s; ++k) {
            const int begin = static_cast<int>(static_cast<long>(k) * chunks / s);
            const int end = static_cast<int>(static_cast<long>(k + 1) * chunks / s);
            for (std::size_t q = i; q < j; ++q) {
                Item it = items[q];
                if (s > 1) {
                    it.stream.chunk_begin = begin;
                    it.stream.chunk_end = end;
                    it.stream.first_sample = begin > 0 ? dp->chunk_first_block[static_cast<std::size_t>(begin - 1)] : 0;
                }
                out.push_back(it);
            }
        }
        i = j;
    }
    return out;
}

} // namespace

void Executor::Impl::compile(const std::vector<PlaneTask> &tasks, Compiled &out,
                             const std::function<char *(std::size_t)> &scratch, std::uint32_t *status,
                             const Tuning *tuning, int vectors_per_warp) {
    const bool paired = vectors_per_warp ? vectors_per_warp == 64 : allow_paired;
    auto &temporaries = out.temporaries;
    // Per task: which kernels run each pass, and the scratch they need.
    struct Route {
        const DevicePlan *h = nullptr, *v = nullptr;
        bool f64 = false, h_stream = false, v_stream = false;
        // Float32 2D planes keep the intermediate transposed (destination
        // column-major): both passes then read adjacent samples and write
        // adjacent vectors.
        // 2D passes: 0 sequential, 3 chunk-delayed, 4 paired chunk-delayed,
        // 5 two-pass transposing.
        bool transposed = false;
        // Float64 planes whose plans both admit the Float64 two-pass
        // transposing kernels (kind 6): a transposed Float64 intermediate.
        bool transposed64 = false;
        int h_kind = 0, v_kind = 0;
        std::size_t mid = 0, mid_stride = 0, fwd = 0, fwd_stride = 0;
        // Float64 segments per pass (1: whole vectors) and their forward-value
        // scratch (each segment's own, margins included).
        int seg_h = 1, seg_v = 1;
        std::size_t yseg_h = 0, yseg_v = 0;
        // Refinement (f64_refine): per-vector correction scratch of each
        // pass and the Float64 result plane of the columns pass.
        bool refine = false;
        std::size_t ref_h = 0, ref_v = 0, x64 = 0;
    };
    std::vector<Route> routes(tasks.size());
    std::size_t bytes = 0;
    for (std::size_t t = 0; t < tasks.size(); ++t) {
        const auto &task = tasks[t];
        const AxisPlan *h = task.horizontal, *v = task.vertical;
        if (!h && !v) throw std::invalid_argument("plane task without a plan");
        auto &r = routes[t];
        r.h = h ? &device_plan(*h, task.horizontal_keep, temporaries, out.private_uploads) : nullptr;
        r.v = v ? &device_plan(*v, task.vertical_keep, temporaries, out.private_uploads) : nullptr;
        r.f64 = (h && h->requires_float64()) || (v && v->requires_float64());
        if (task.score && r.f64) throw std::invalid_argument("fused scoring needs Float32 plans");
        if (!r.f64 && allow_stream) {
            r.h_stream = r.h && stream_row_ok(*r.h, h && v ? task.sample : dev::Sample::f32);
            r.v_stream = r.v && r.v->stream;
        }
        const std::size_t es = r.f64 ? 8 : 4;
        if (h && v && r.f64 && allow_stream && r.h->stream64 && r.v->stream64) {
            r.transposed64 = true;
            r.mid_stride = (static_cast<std::size_t>(v->source_size) + 1) / 2 * 2;
            r.mid = bytes;
            bytes += align_up(r.mid_stride * static_cast<std::size_t>(h->destination_size) * 8);
            r.fwd_stride = static_cast<std::size_t>(h->destination_size);
            r.fwd = bytes;
            bytes += align_up(r.fwd_stride * static_cast<std::size_t>(v->destination_size) * 8);
            if (f64_refine) {
                r.refine = true;
                r.ref_h = bytes;
                bytes += align_up(r.mid_stride * static_cast<std::size_t>(h->destination_size) * 8);
                r.x64 = bytes;
                bytes += align_up(r.fwd_stride * static_cast<std::size_t>(v->destination_size) * 8);
                r.ref_v = bytes;
                bytes += align_up(r.fwd_stride * static_cast<std::size_t>(v->destination_size) * 8);
            }
        } else if (h && v && !r.f64) {
            r.transposed = true;
            auto pass_kind = [&](const DevicePlan &dp) {
                if (!allow_stream) return 0;
                const bool delayed = dp.stream && dp.stream_t;
                if (dp.stream_x && (prefer_exact || !delayed)) return 5;
                if (delayed) return paired && dp.stream_p ? 4 : 3;
                return 0;
            };
            r.h_kind = pass_kind(*r.h);
            r.v_kind = pass_kind(*r.v);
            if (task.score) {
                // The fused scoring pass replaces the chunk-delayed one.
                if (fused_window(*r.v) < 0 || task.sample != dev::Sample::f32)
                    throw std::invalid_argument("fused scoring needs a chunk-delayed Float32 columns pass");
                r.v_kind = 9;
            }
            r.mid_stride = (static_cast<std::size_t>(v->source_size) + 3) / 4 * 4;
            r.mid = bytes;
            bytes += align_up(r.mid_stride * static_cast<std::size_t>(h->destination_size) * 4);
            // Forward values of the second pass when the output cannot hold
            // them (integer samples): the sequential and two-pass kernels.
            if ((r.v_kind == 0 || r.v_kind == 5) && task.sample != dev::Sample::f32) {
                r.fwd_stride = static_cast<std::size_t>(h->destination_size);
                r.fwd = bytes;
                bytes += align_up(r.fwd_stride * static_cast<std::size_t>(v->destination_size) * 4);
            }
        } else if (h && v) {
            r.mid_stride = static_cast<std::size_t>(h->destination_size);
            r.mid = bytes;
            bytes += align_up(r.mid_stride * static_cast<std::size_t>(v->source_size) * es);
            if (r.f64 || (!r.v_stream && task.sample != dev::Sample::f32)) {
                r.fwd_stride = static_cast<std::size_t>(h->destination_size);
                r.fwd = bytes;
                bytes += align_up(r.fwd_stride * static_cast<std::size_t>(v->destination_size) * es);
            }
        } else if (r.f64) {
            const AxisPlan *p = h ? h : v;
            r.fwd_stride = h ? static_cast<std::size_t>(p->destination_size) : static_cast<std::size_t>(task.vectors);
            const std::size_t lines = h ? static_cast<std::size_t>(task.vectors) : static_cast<std::size_t>(p->destination_size);
            r.fwd = bytes;
            bytes += align_up(r.fwd_stride * lines * 8);
        }
    }
    // Float64 segments: each pass's kind-6 warps decide the split (as for the
    // chunk-delayed kernels); every segment writes its forward values, its
    // margins included, to a scratch region of its own.
    // The two-pass Float32 kernels (kind 5) split alike, with their own
    // margins and Float32 forward values.
    {
        long warps64[2] = {0, 0}, warps32[2] = {0, 0};
        for (std::size_t t = 0; t < tasks.size(); ++t) {
            const auto &r = routes[t];
            if (r.transposed64) {
                warps64[0] += (tasks[t].vertical->source_size + 31) / 32;
                warps64[1] += (tasks[t].horizontal->destination_size + 31) / 32;
            }
            if (r.transposed && r.h_kind == 5) warps32[0] += (tasks[t].vertical->source_size + 31) / 32;
            if (r.transposed && r.v_kind == 5) warps32[1] += (tasks[t].horizontal->destination_size + 31) / 32;
        }
        auto split32 = [&](const DevicePlan &dp, int destinations, long warps) {
            if (!dp.exact_margin || segment_mode == 1) return 1;
            const int chunks = (destinations + kStreamChunk - 1) / kStreamChunk;
            int s = segment_mode >= 2 ? segment_mode
                                      : (warps > 0 ? static_cast<int>(std::min<long>(warp_slots / (2 * warps), 64)) : 1);
            return std::max(1, std::min(s, chunks / (2 * dp.exact_margin + 1)));
        };
        for (std::size_t t = 0; t < tasks.size(); ++t) {
            auto &r = routes[t];
            if (!r.transposed) continue;
            const AxisPlan *h = tasks[t].horizontal, *v = tasks[t].vertical;
            if (r.h_kind == 5 && (r.seg_h = split32(*r.h, h->destination_size, warps32[0])) > 1) {
                r.yseg_h = bytes;
                bytes += align_up(segment64_chunks(h->destination_size, r.seg_h, r.h->exact_margin) * kStreamChunk
                                  * r.mid_stride * 4);
            }
            if (r.v_kind == 5 && (r.seg_v = split32(*r.v, v->destination_size, warps32[1])) > 1) {
                r.yseg_v = bytes;
                bytes += align_up(segment64_chunks(v->destination_size, r.seg_v, r.v->exact_margin) * kStreamChunk
                                  * static_cast<std::size_t>(h->destination_size) * 4);
            }
        }
        auto split = [&](const DevicePlan &dp, int destinations, long warps) {
            if (!dp.stream64_seg || segment_mode == 1) return 1;
            const int chunks = (destinations + kStreamChunk - 1) / kStreamChunk;
            // Margins cost 2 x margin chunks a boundary: split only launches
            // that fill less than half of the GPU's warp slots.
            int s = segment_mode >= 2 ? segment_mode
                                      : (warps > 0 ? static_cast<int>(std::min<long>(warp_slots / (2 * warps), 64)) : 1);
            return std::max(1, std::min(s, chunks / (2 * dp.margin64)));
        };
        for (std::size_t t = 0; t < tasks.size(); ++t) {
            auto &r = routes[t];
            if (!r.transposed64) continue;
            const AxisPlan *h = tasks[t].horizontal, *v = tasks[t].vertical;
            r.seg_h = split(*r.h, h->destination_size, warps64[0]);
            if (r.seg_h > 1) {
                r.yseg_h = bytes;
                bytes += align_up(segment64_chunks(h->destination_size, r.seg_h, r.h->margin64) * kStreamChunk
                                  * r.mid_stride * 8);
            }
            r.seg_v = split(*r.v, v->destination_size, warps64[1]);
            if (r.seg_v > 1) {
                r.yseg_v = bytes;
                bytes += align_up(segment64_chunks(v->destination_size, r.seg_v, r.v->margin64) * kStreamChunk
                                  * r.fwd_stride * 8);
            }
        }
    }
    out.scratch_bytes = bytes;
    char *base = scratch(std::max<std::size_t>(bytes, kAlign));

    struct Item {
        dev::AxisJob axis{};
        dev::StreamJob stream{};
        std::uint64_t bytes = 0;
        const DevicePlan *plan = nullptr;   // chunk-delayed transposing passes
        int tiles = 0;                      // fused scoring: CTAs of the job
    };
    std::map<GroupKey, std::vector<Item>> groups;
    for (std::size_t t = 0; t < tasks.size(); ++t) {
        const auto &task = tasks[t];
        const auto &r = routes[t];
        const AxisPlan *h = task.horizontal, *v = task.vertical;
        const dev::Conversion conv = to_dev(task.conversion);
        const dev::Sample mid_kind = r.f64 ? dev::Sample::f64 : dev::Sample::f32;
        const int seq_kind = r.f64 ? 1 : 0;
        if (r.transposed64) {
            void *mid = base + r.mid;
            const auto pitch = static_cast<std::int64_t>(r.mid_stride);
            Item hi, vi;
            hi.bytes = static_cast<std::uint64_t>(v->source_size) * h->source_size * sample_bytes(task.sample);
            vi.bytes = static_cast<std::uint64_t>(h->destination_size) * v->destination_size
                * sample_bytes(task.sample);
            auto &a = hi.stream;
            a.plan = r.h->stream_view64;
            a.in = task.input; a.in_elem = 1; a.in_vec = task.input_stride;
            a.out = mid; a.out_elem = pitch; a.out_vec = 1;
            a.y = static_cast<float *>(mid); a.y_elem = pitch;   // Float64 forward values in place
            a.vectors = v->source_size;
            a.conv = conv;
            push_segments(groups[{0, 6, h->half_bandwidth, task.sample, dev::Sample::f64, 0}], hi,
                          r.h->chunk_first_block64, r.h->margin64, h->destination_size, r.seg_h, base + r.yseg_h, pitch,
                          8);
            const auto xs = static_cast<std::int64_t>(r.fwd_stride);
            if (r.refine) {
                // Rows: x is the intermediate (destination-major), b the input.
                Item ri;
                auto &q = ri.axis;
                q.plan = r.h->view;
                q.in = task.input; q.in_elem = 1; q.in_vec = task.input_stride;
                q.out = mid; q.out_elem = pitch; q.out_vec = 1;
                q.fwd = base + r.ref_h; q.fwd_elem = pitch; q.fwd_vec = 1;
                q.vectors = v->source_size;
                q.conv = conv;
                groups[{0, 7, h->half_bandwidth, task.sample, dev::Sample::f64, 0}].push_back(ri);
            }
            auto &b = vi.stream;
            b.plan = r.v->stream_view64;
            b.in = mid; b.in_elem = 1; b.in_vec = pitch;
            if (r.refine) {
                b.out = base + r.x64; b.out_elem = xs; b.out_vec = 1;
            } else {
                b.out = task.output; b.out_elem = task.output_stride; b.out_vec = 1;
            }
            b.y = reinterpret_cast<float *>(base + r.fwd); b.y_elem = xs;
            b.vectors = h->destination_size;
            b.conv = conv;
            push_segments(groups[{1, 6, v->half_bandwidth, dev::Sample::f64, r.refine ? dev::Sample::f64 : task.sample,
                                  0}], vi,
                          r.v->chunk_first_block64, r.v->margin64, v->destination_size, r.seg_v, base + r.yseg_v, xs, 8);
            if (r.refine) {
                // Columns: x is the Float64 result plane, b the intermediate;
                // then the conversion into the output.
                Item ci, oi;
                auto &q = ci.axis;
                q.plan = r.v->view;
                q.in = mid; q.in_elem = 1; q.in_vec = pitch;
                q.out = base + r.x64; q.out_elem = xs; q.out_vec = 1;
                q.fwd = base + r.ref_v; q.fwd_elem = xs; q.fwd_vec = 1;
                q.vectors = h->destination_size;
                q.conv = conv;
                groups[{1, 7, v->half_bandwidth, dev::Sample::f64, dev::Sample::f64, 0}].push_back(ci);
                auto &o = oi.axis;
                o.plan = r.h->view;                 // destination_size: the row length
                o.in = base + r.x64; o.in_elem = 1; o.in_vec = xs;
                o.out = task.output; o.out_elem = 1; o.out_vec = task.output_stride;
                o.vectors = v->destination_size;
                o.conv = conv;
                groups[{1, 8, 0, dev::Sample::f64, task.sample, 0}].push_back(oi);
            }
            continue;
        }
        if (r.transposed) {
            float *mid = reinterpret_cast<float *>(base + r.mid);
            const auto pitch = static_cast<std::int64_t>(r.mid_stride);
            Item hi, vi;
            hi.bytes = static_cast<std::uint64_t>(v->source_size) * h->source_size * sample_bytes(task.sample);
            vi.bytes = static_cast<std::uint64_t>(h->destination_size) * v->destination_size
                * sample_bytes(task.sample);
            if (r.h_kind) {
                auto &j = hi.stream;
                j.plan = r.h_kind == 4 ? r.h->stream_view2
                       : r.h_kind == 3 && r.h->stream_union ? r.h->stream_view_g : r.h->stream_view;
                j.in = task.input; j.in_elem = 1; j.in_vec = task.input_stride;
                j.out = mid; j.out_elem = pitch; j.out_vec = 1;
                j.y = mid; j.y_elem = pitch;                // forward values in place
                j.vectors = v->source_size;
                j.conv = conv;
                hi.plan = r.h;
                auto &group = groups[{0, r.h_kind, h->half_bandwidth, task.sample, dev::Sample::f32,
                                      compiled_window(*r.h, r.h_kind)}];
                if (r.h_kind == 5)
                    push_segments(group, hi, r.h->chunk_first_block, r.h->exact_margin, h->destination_size, r.seg_h,
                                  base + r.yseg_h, pitch, 4);
                else
                    group.push_back(hi);
            } else {
                auto &j = hi.axis;
                j.plan = r.h->view;
                j.in = task.input; j.in_elem = 1; j.in_vec = task.input_stride;
                j.out = mid; j.out_elem = pitch; j.out_vec = 1;
                j.fwd = mid; j.fwd_elem = pitch; j.fwd_vec = 1;
                j.vectors = v->source_size;
                j.conv = conv;
                groups[{0, 0, h->half_bandwidth, task.sample, dev::Sample::f32}].push_back(hi);
            }
            if (r.v_kind == 9) {
                auto &j = vi.stream;
                j.plan = r.v->stream_union ? r.v->stream_view_g : r.v->stream_view;
                j.in = mid; j.in_elem = 1; j.in_vec = pitch;
                j.vectors = h->destination_size;
                j.conv = conv;
                j.score = task.score;
                vi.plan = r.v;
                vi.tiles = task.score_tiles;
                vi.bytes = static_cast<std::uint64_t>(h->destination_size) * v->source_size * 4;
                groups[{1, 9, v->half_bandwidth, dev::Sample::f32, dev::Sample::f32, fused_window(*r.v)}].push_back(vi);
            } else if (r.v_kind) {
                auto &j = vi.stream;
                j.plan = r.v_kind == 4 ? r.v->stream_view2
                       : r.v_kind == 3 && r.v->stream_union ? r.v->stream_view_g : r.v->stream_view;
                j.in = mid; j.in_elem = 1; j.in_vec = pitch;
                j.out = task.output; j.out_elem = task.output_stride; j.out_vec = 1;
                if (r.fwd_stride) {
                    j.y = reinterpret_cast<float *>(base + r.fwd);
                    j.y_elem = static_cast<std::int64_t>(r.fwd_stride);
                } else {
                    j.y = static_cast<float *>(task.output);   // Float32 output: in place
                    j.y_elem = task.output_stride;
                }
                j.vectors = h->destination_size;
                j.conv = conv;
                vi.plan = r.v;
                auto &group = groups[{1, r.v_kind, v->half_bandwidth, dev::Sample::f32, task.sample,
                                      compiled_window(*r.v, r.v_kind)}];
                if (r.v_kind == 5)
                    push_segments(group, vi, r.v->chunk_first_block, r.v->exact_margin, v->destination_size, r.seg_v,
                                  base + r.yseg_v, static_cast<std::int64_t>(h->destination_size), 4);
                else
                    group.push_back(vi);
            } else {
                auto &j = vi.axis;
                j.plan = r.v->view;
                j.in = mid; j.in_elem = 1; j.in_vec = pitch;
                j.out = task.output; j.out_elem = task.output_stride; j.out_vec = 1;
                if (r.fwd_stride) {
                    j.fwd = base + r.fwd; j.fwd_elem = static_cast<std::int64_t>(r.fwd_stride); j.fwd_vec = 1;
                } else {
                    j.fwd = task.output; j.fwd_elem = task.output_stride; j.fwd_vec = 1;
                }
                j.vectors = h->destination_size;
                j.conv = conv;
                groups[{1, 0, v->half_bandwidth, dev::Sample::f32, task.sample}].push_back(vi);
            }
            continue;
        }
        if (h) {
            // Rows: source rows of the input, into the intermediate (2D) or
            // the output (rows only).
            const void *in = task.input;
            const std::int64_t in_vec = task.input_stride;
            void *out = v ? static_cast<void *>(base + r.mid) : task.output;
            const std::int64_t out_vec = v ? static_cast<std::int64_t>(r.mid_stride) : task.output_stride;
            const int vectors = v ? v->source_size : task.vectors;
            const dev::Sample out_kind = v ? mid_kind : task.sample;
            Item it;
            it.bytes = static_cast<std::uint64_t>(vectors) * h->source_size * sample_bytes(task.sample);
            if (!v) it.bytes += static_cast<std::uint64_t>(vectors) * h->destination_size * 4;
            if (r.h_stream) {
                auto &j = it.stream;
                j.plan = r.h->stream_view;
                j.in = in; j.in_elem = 1; j.in_vec = in_vec;
                j.out = out; j.out_elem = 1; j.out_vec = out_vec;
                j.vectors = vectors;
                j.conv = conv;
                groups[{0, 2, h->half_bandwidth, task.sample, out_kind}].push_back(it);
            } else {
                auto &j = it.axis;
                j.plan = r.h->view;
                j.in = in; j.in_elem = 1; j.in_vec = in_vec;
                j.out = out; j.out_elem = 1; j.out_vec = out_vec;
                if (!v && r.f64) {
                    j.fwd = base + r.fwd; j.fwd_elem = 1; j.fwd_vec = static_cast<std::int64_t>(r.fwd_stride);
                } else {
                    j.fwd = out; j.fwd_elem = 1; j.fwd_vec = out_vec;
                }
                j.vectors = vectors;
                j.conv = conv;
                groups[{0, seq_kind, h->half_bandwidth, task.sample, out_kind}].push_back(it);
            }
        }
        if (v) {
            // Columns: destination columns of the intermediate (2D) or of the
            // input (columns only), into the output.
            const void *in = h ? static_cast<const void *>(base + r.mid) : task.input;
            const std::int64_t in_elem = h ? static_cast<std::int64_t>(r.mid_stride) : task.input_stride;
            const int vectors = h ? h->destination_size : task.vectors;
            const dev::Sample in_kind = h ? mid_kind : task.sample;
            Item it;
            it.bytes = static_cast<std::uint64_t>(vectors) * v->destination_size * sample_bytes(task.sample);
            if (!h) it.bytes += static_cast<std::uint64_t>(vectors) * v->source_size * 4;
            if (r.v_stream) {
                auto &j = it.stream;
                j.plan = r.v->stream_view;
                j.in = in; j.in_elem = in_elem; j.in_vec = 1;
                j.out = task.output; j.out_elem = task.output_stride; j.out_vec = 1;
                j.vectors = vectors;
                j.conv = conv;
                groups[{1, 2, v->half_bandwidth, in_kind, task.sample}].push_back(it);
            } else {
                auto &j = it.axis;
                j.plan = r.v->view;
                j.in = in; j.in_elem = in_elem; j.in_vec = 1;
                j.out = task.output; j.out_elem = task.output_stride; j.out_vec = 1;
                if (r.fwd_stride) {
                    j.fwd = base + r.fwd; j.fwd_elem = static_cast<std::int64_t>(r.fwd_stride); j.fwd_vec = 1;
                } else {
                    j.fwd = task.output; j.fwd_elem = task.output_stride; j.fwd_vec = 1;
                }
                j.vectors = vectors;
                j.conv = conv;
                groups[{1, seq_kind, v->half_bandwidth, in_kind, task.sample}].push_back(it);
            }
        }
    }

    // One job table for every group: AxisJob and StreamJob records share a
    // byte buffer, each group's records contiguous and 256-byte aligned.
    const int stream_block = stream_threads();
    std::vector<Launch> &launches = out.launches;
    std::vector<char> &table = out.table;
    table.clear();
    launches.clear();
    for (auto &[key, items] : groups) {
        const bool fused = key.kind == 9;
        const bool is_stream = (key.kind >= 2 && key.kind <= 6) || fused;
        int per_block = key.kind == 2 ? stream_block : fused ? kScoreCtaThreads
                      : is_stream ? tstream_threads : kSeqThreads;
        if (tuning && key.kind != 2 && key.kind <= 6) {
            const GroupTuple g{key.pass, key.kind, key.hb, static_cast<int>(key.in), static_cast<int>(key.out),
                               key.variant};
            if (auto it = tuning->find(g); it != tuning->end()) per_block = it->second;
        }
        const std::size_t rec = is_stream ? sizeof(dev::StreamJob) : sizeof(dev::AxisJob);
        int blocks = 0, count = 0, record_floats = 0;
        std::uint64_t bytes_moved = 0;
        const std::size_t offset = align_up(table.size());
        table.resize(offset);
        // Transposing kernels are assigned warps, not CTAs: a CTA's warps
        // may serve consecutive jobs of one plan (they share the CTA's record
        // copies), so only plan changes round up to a whole CTA.
        const bool by_warp = (key.kind >= 3 && key.kind <= 6) || fused;
        const int warps_per_cta = per_block / 32;
        const int vectors_per_warp = key.kind == 4 ? 64 : 32;
        // Jobs of one plan stay together (they share record copies); plans
        // with the longest vectors come first, so that the CTAs that take
        // longest start in the first wave and the launch's tail is short
        // (longest-first list scheduling).
        if (by_warp)
            std::stable_sort(items.begin(), items.end(), [](const Item &a, const Item &b) {
                const int na = a.stream.plan.destination_size, nb = b.stream.plan.destination_size;
                if (na != nb) return na > nb;
                return a.stream.plan.forward < b.stream.plan.forward;
            });
        if (key.kind == 3) items = segment_items(items, vectors_per_warp, segment_mode, warp_slots);
        int warps = 0;
        const float *run_plan = nullptr;
        int run_chunk = 0;
        for (auto &it : items) {
            const int vectors = is_stream ? it.stream.vectors : it.axis.vectors;
            if (vectors <= 0) continue;
            if (fused) {
                // One CTA per tile; every job starts on a CTA.
                warps = (warps + warps_per_cta - 1) / warps_per_cta * warps_per_cta;
                it.stream.first_block = warps;
                warps += it.tiles * warps_per_cta;
                blocks = warps / warps_per_cta;
            } else if (by_warp) {
                if (warps && (it.stream.plan.forward != run_plan || it.stream.chunk_begin != run_chunk))
                    warps = (warps + warps_per_cta - 1) / warps_per_cta * warps_per_cta;
                run_plan = it.stream.plan.forward;
                run_chunk = it.stream.chunk_begin;
                it.stream.first_block = warps;     // first warp of the job
                warps += (vectors + vectors_per_warp - 1) / vectors_per_warp;
                blocks = (warps + warps_per_cta - 1) / warps_per_cta;
            } else {
                if (is_stream) it.stream.first_block = blocks; else it.axis.first_block = blocks;
                blocks += (vectors + per_block - 1) / per_block;
            }
            bytes_moved += it.bytes;
            if (is_stream) {
                it.stream.status = status;
                it.stream.feed_stall_test = feed_stall_test ? 1 : 0;
            }
            if (is_stream)
                record_floats = std::max(record_floats, it.stream.plan.forward_stride + it.stream.plan.backward_stride);
            const char *src = is_stream ? reinterpret_cast<const char *>(&it.stream)
                                        : reinterpret_cast<const char *>(&it.axis);
            table.insert(table.end(), src, src + rec);
            ++count;
        }
        if (count)
            launches.push_back({key.pass, key.kind, key.hb, key.in, key.out, key.variant, offset, count, blocks,
                                bytes_moved, record_floats, per_block});
    }
    out.tasks = tasks.size();
}

void Executor::Impl::launch(const Compiled &c, const char *device_table, cudaStream_t stream,
                            std::uint32_t *status) {
    for (const auto &l : c.launches) {
        Record *rec = nullptr;
        cudaStreamCaptureStatus capturing = cudaStreamCaptureStatusNone;
        cudaStreamIsCapturing(stream, &capturing);
        if (profiling && capturing == cudaStreamCaptureStatusNone) {
            std::scoped_lock lock(mutex);
            records.emplace_back();
            rec = &records.back();
            rec->name = kernel_name({l.pass, l.kind, l.hb, l.in, l.out, l.variant});
            rec->bytes = l.bytes;
            rec->start = pooled_event();
            rec->stop = pooled_event();
            cuda_check(cudaEventRecord(rec->start, stream), "recording event");
        }
        const char *dev_table = device_table + l.offset;
        int rc = 0;
        if (l.kind == 9) {
            rc = launch_tscore(reinterpret_cast<const dev::StreamJob *>(dev_table), l.count, l.blocks, l.hb,
                               l.variant, l.record_floats, stream);
        } else if (l.kind == 7) {
            rc = launch_refine64(reinterpret_cast<const dev::AxisJob *>(dev_table), l.count, l.blocks, l.threads,
                                 l.hb, l.in, status, stream);
        } else if (l.kind == 8) {
            rc = launch_convert64(reinterpret_cast<const dev::AxisJob *>(dev_table), l.count, l.blocks, l.threads,
                                  l.out, status, stream);
        } else if (l.kind == 6) {
            rc = launch_tsolve64(reinterpret_cast<const dev::StreamJob *>(dev_table), l.count, l.blocks, l.threads,
                                 l.hb, l.in, l.out, l.record_floats, f64_fused, status, stream);
        } else if (l.kind == 5) {
            rc = launch_tsolve(reinterpret_cast<const dev::StreamJob *>(dev_table), l.count, l.blocks, l.threads,
                               l.hb, l.variant ? 8 : 0, l.in, l.out, l.record_floats, stream);
        } else if (l.kind == 4) {
            rc = launch_tstream2(reinterpret_cast<const dev::StreamJob *>(dev_table), l.count, l.blocks,
                                 l.threads, l.hb, l.variant ? 8 : 0, l.in, l.out, l.record_floats, stream);
        } else if (l.kind == 3) {
            rc = launch_tstream(reinterpret_cast<const dev::StreamJob *>(dev_table), l.count, l.blocks,
                                l.threads, l.hb, l.variant, l.in, l.out, l.record_floats,
                                stream);
        } else if (l.kind == 2) {
            rc = launch_stream(reinterpret_cast<const dev::StreamJob *>(dev_table), l.count, l.blocks,
                               l.hb, kStreamChunk, l.pass == 0, l.in, l.out, l.record_floats,
                               stream);
        } else if (l.kind == 1) {
            rc = launch_axis_f64(reinterpret_cast<const dev::AxisJob *>(dev_table), l.count, l.blocks,
                                 l.threads, l.hb, l.in, l.out, status, stream);
        } else {
            rc = launch_axis_f32(reinterpret_cast<const dev::AxisJob *>(dev_table), l.count, l.blocks,
                                 l.threads, l.hb, l.in, l.out, stream);
        }
        cuda_check(rc, "launching axis kernel");
        if (rec) cuda_check(cudaEventRecord(rec->stop, stream), "recording event");
    }
    std::scoped_lock lock(mutex);
    stats.launches += c.launches.size();
    stats.plane_tasks += c.tasks;
}

namespace {

bool same_task(const PlaneTask &a, const PlaneTask &b) {
    const auto &x = a.conversion, &y = b.conversion;
    return a.horizontal == b.horizontal && a.vertical == b.vertical && a.input == b.input
        && a.input_stride == b.input_stride && a.output == b.output && a.output_stride == b.output_stride
        && a.sample == b.sample && a.vectors == b.vectors && a.horizontal_keep == b.horizontal_keep
        && a.vertical_keep == b.vertical_keep && a.score == b.score && a.score_tiles == b.score_tiles
        && x.input_offset == y.input_offset && x.input_scale == y.input_scale && x.output_scale == y.output_scale
        && x.output_offset == y.output_offset && x.output_maximum == y.output_maximum;
}

} // namespace

void Executor::Impl::enqueue(Workspace &ws, const std::vector<PlaneTask> &tasks, char *scratch,
                             std::size_t scratch_capacity, cudaStream_t copies) {
    // A call that repeats one of the workspace's recent task lists (a frame
    // server's next frame through the same slot) reuses its compiled launches.
    auto hit = ws.compiled.end();
    if (!scratch) {
        hit = std::find_if(ws.compiled.begin(), ws.compiled.end(), [&](const Workspace::CompiledEntry &e) {
            return e.scratch == ws.scratch.data() && e.tasks.size() == tasks.size()
                && std::equal(tasks.begin(), tasks.end(), e.tasks.begin(), same_task);
        });
    }
    std::shared_ptr<Compiled> held;
    const char *device_table = nullptr;
    if (hit != ws.compiled.end()) {
        held = std::static_pointer_cast<Compiled>(hit->compiled);
        std::rotate(ws.compiled.begin(), hit, hit + 1);
        device_table = ws.compiled.front().table->data();
        std::scoped_lock lock(mutex);
        ++stats.compile_reuses;
    } else {
        held = std::make_shared<Compiled>();
        compile(tasks, *held, [&](std::size_t bytes) {
            if (scratch) {
                if (bytes > scratch_capacity) throw std::length_error("batch scratch exceeds the caller's buffer");
                return scratch;
            }
            ws.scratch.reserve(bytes);
            return ws.scratch.data();
        }, ws.status);
        // Only task lists whose plans all stay resident (prepared, or cached
        // with their owners) are kept: a private upload is for one call.  A
        // compile may have moved the scratch: entries on the old one go.
        if (!scratch) {
            char *now = ws.scratch.data();
            ws.compiled.erase(std::remove_if(ws.compiled.begin(), ws.compiled.end(),
                                             [now](const Workspace::CompiledEntry &e) { return e.scratch != now; }),
                              ws.compiled.end());
            if (held->private_uploads == 0 && !held->launches.empty()) {
                // The least recent entry's table buffer is reused (freeing
                // device memory would wait for the whole device).
                std::unique_ptr<DeviceBuffer> table;
                if (ws.compiled.size() >= Workspace::kCompiledEntries) {
                    table = std::move(ws.compiled.back().table);
                    ws.compiled.pop_back();
                }
                if (!table) table = std::make_unique<DeviceBuffer>();
                ws.copy_table(*table, held->table, copies);
                ws.compiled.insert(ws.compiled.begin(), Workspace::CompiledEntry{held, tasks, now, std::move(table)});
                device_table = ws.compiled.front().table->data();
            }
        }
    }
    const Compiled &c = *held;
    if (!device_table && !c.launches.empty()) {
        ws.upload_table(c.table, copies);
        device_table = ws.jobs.data();
    }
    if (copies) ws.follow(copies);
    if (c.launches.empty()) return;
    launch(c, device_table, ws.stream, ws.status);
    // Float64 kernels report non-finite data, the transposing kernels a
    // stalled feed.
    for (const auto &l : c.launches) ws.status_pending |= l.kind == 1 || l.kind >= 3;
    if (c.private_uploads > 0) {
        // Private plan uploads must outlive the kernels that read them.
        // (Cached plans evicted meanwhile are released by cudaFree, which
        // waits for the work in flight.)
        cuda_check(cudaStreamSynchronize(ws.stream), "synchronizing");
    }
}

namespace {

// The error a nonzero device status word stands for.
[[noreturn]] void throw_status(std::uint32_t status) {
    if (status & dev::kStatusFeedStall)
        throw std::runtime_error("a transposing kernel's feed wait ran out (its outputs are not valid)");
    if (status & dev::kStatusNonFiniteInput) throw std::runtime_error("Float64 input contains NaN or infinity");
    throw std::runtime_error("Float64 execution produced NaN or infinity");
}

} // namespace

void Executor::Impl::finish(Workspace &ws) {
    if (!ws.status_pending) {
        // Only the Float64 and transposing kernels set the status word:
        // nothing to read.
        cuda_check(cudaStreamSynchronize(ws.stream), "synchronizing");
        return;
    }
    ws.status_pending = false;
    cuda_check(cudaStreamSynchronize(ws.stream), "synchronizing");
    const std::uint32_t status = *static_cast<volatile std::uint32_t *>(ws.status_host);
    if (status) {
        *static_cast<volatile std::uint32_t *>(ws.status_host) = 0;
        throw_status(status);
    }
}

Executor::Executor(int device) : impl_(std::make_unique<Impl>()) {
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0)
        throw std::runtime_error("backend 'cuda' requires an available CUDA device");
    if (device < 0) cuda_check(cudaGetDevice(&device), "querying device");
    if (device >= count) throw std::invalid_argument("CUDA device index out of range");
    impl_->device = device;
    if (const char *env = std::getenv("DSMVC_GB_STREAM"); env && std::string(env) == "0")
        impl_->allow_stream = false;
    if (const char *env = std::getenv("DSMVC_GB_PAIRED"))
        impl_->allow_paired = std::string(env) == "1";
    if (const char *env = std::getenv("DSMVC_GB_EXACT"))
        impl_->prefer_exact = std::string(env) == "1";
    if (impl_->prefer_exact) impl_->f64_fused = false;
    if (const char *env = std::getenv("DSMVC_GB_F64_EXACT"))
        impl_->f64_fused = std::string(env) != "1" && !impl_->prefer_exact;
    if (const char *env = std::getenv("DSMVC_GB_F64_REFINE")) impl_->f64_refine = std::string(env) == "1";
    if (const char *env = std::getenv("DSMVC_GB_HOST_DIRECT")) impl_->host_direct = std::string(env) == "1";
    if (const char *env = std::getenv("DSMVC_GB_FEED_STALL_TEST")) impl_->feed_stall_test = std::string(env) == "1";
    if (const char *env = std::getenv("DSMVC_GB_PIPELINE_MB")) {
        char *end = nullptr;
        const long v = std::strtol(env, &end, 10);
        if (end && *end == '\0' && v >= 1 && v <= 65536) impl_->pipe_group_bytes = static_cast<std::size_t>(v) << 20;
    }
    if (const char *env = std::getenv("DSMVC_GB_TSTREAM_THREADS")) {
        char *end = nullptr;
        const long v = std::strtol(env, &end, 10);
        if (end && *end == '\0' && v >= 32 && v <= 256 && v % 32 == 0) impl_->tstream_threads = static_cast<int>(v);
    }
    if (const char *env = std::getenv("DSMVC_GB_SEGMENTS")) {
        char *end = nullptr;
        const long v = std::strtol(env, &end, 10);
        if (end && *end == '\0' && v >= 0 && v <= 1024) impl_->segment_mode = static_cast<int>(v);
    }
    {
        int sms = 0;
        cuda_check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device), "querying SMs");
        impl_->warp_slots = sms * kTResidentWarps;
    }
    if (const char *env = std::getenv("DSMVC_GB_PLAN_CACHE_MB")) {
        char *end = nullptr;
        const long v = std::strtol(env, &end, 10);
        if (end && *end == '\0' && v >= 16 && v <= 4096)
            impl_->cache_capacity = static_cast<std::size_t>(v) << 20;
    }
    if (const char *env = std::getenv("DSMVC_GB_STREAMS")) {
        char *end = nullptr;
        const long v = std::strtol(env, &end, 10);
        if (end && *end == '\0' && v >= 1 && v <= 16) impl_->max_slots = static_cast<std::size_t>(v);
    }
    DeviceGuard guard(device);
    cuda_check(cudaFree(nullptr), "initialising the primary context");
}

Executor::~Executor() {
    if (!impl_) return;
    DeviceGuard guard(impl_->device);
    impl_->slots.clear();
    impl_->stream_spaces.clear();
    impl_->plans.clear();
    for (auto e : impl_->event_pool) cudaEventDestroy(e);
}

int Executor::device() const noexcept { return impl_->device; }

void Executor::prepare(std::shared_ptr<const AxisPlan> plan) {
    if (!plan || !plan->valid()) throw std::invalid_argument("cannot prepare an invalid axis plan");
    {
        std::scoped_lock lock(impl_->mutex);
        if (impl_->plans.count(plan.get())) return;
        if (impl_->sealed) throw std::logic_error("executor is sealed; prepare plans before seal()");
    }
    DeviceGuard guard(impl_->device);
    auto dp = upload_plan(*plan, plan);
    std::scoped_lock lock(impl_->mutex);
    impl_->stats.plan_uploads += 1;
    impl_->stats.device_plan_bytes += dp->bytes;
    impl_->plans.emplace(plan.get(), std::move(dp));
}

void Executor::prepare_many(const std::vector<std::shared_ptr<const AxisPlan>> &plans) {
    std::vector<std::shared_ptr<const AxisPlan>> fresh;
    {
        std::scoped_lock lock(impl_->mutex);
        for (const auto &p : plans) {
            if (!p) throw std::invalid_argument("cannot prepare a null plan");
            if (impl_->plans.count(p.get())) continue;
            if (impl_->sealed) throw std::logic_error("executor is sealed; prepare plans before seal()");
            fresh.push_back(p);
        }
    }
    std::sort(fresh.begin(), fresh.end());
    fresh.erase(std::unique(fresh.begin(), fresh.end()), fresh.end());
    if (fresh.empty()) return;
    DeviceGuard guard(impl_->device);
    auto uploaded = upload_plans(fresh);
    std::scoped_lock lock(impl_->mutex);
    for (auto &dp : uploaded) {
        if (impl_->plans.count(dp->keep.get())) continue;
        impl_->stats.plan_uploads += 1;
        impl_->stats.device_plan_bytes += dp->bytes;
        const AxisPlan *key = dp->keep.get();
        impl_->plans.emplace(key, std::move(dp));
    }
}

void Executor::seal() {
    std::scoped_lock lock(impl_->mutex);
    impl_->sealed = true;
}

namespace {

void check_rows(const AxisPlan &plan, const void *in, std::ptrdiff_t is, const void *out,
                std::ptrdiff_t os, std::int32_t rows) {
    if (!plan.valid() || !in || !out || is < plan.source_size || os < plan.destination_size || rows < 0)
        throw std::invalid_argument("invalid row executor arguments");
}

void check_columns(const AxisPlan &plan, const void *in, std::ptrdiff_t is, const void *out,
                   std::ptrdiff_t os, std::int32_t columns) {
    if (!plan.valid() || !in || !out || columns < 0 || is < columns || os < columns)
        throw std::invalid_argument("invalid column executor arguments");
}

} // namespace

void Executor::inverse_rows(const AxisPlan &plan, const float *input, std::ptrdiff_t is,
                            float *output, std::ptrdiff_t os, std::int32_t rows,
                            const std::shared_ptr<const AxisPlan> &keep) {
    check_rows(plan, input, is, output, os, rows);
    if (rows == 0) return;
    DeviceGuard guard(impl_->device);
    std::size_t slot = 0;
    Workspace &ws = impl_->acquire_slot(slot);
    try {
        const std::size_t in_bytes = align_up(static_cast<std::size_t>(rows) * plan.source_size * 4);
        const std::size_t out_bytes = align_up(static_cast<std::size_t>(rows) * plan.destination_size * 4);
        ws.staging.reserve(in_bytes + out_bytes);
        char *din = ws.staging.data();
        char *dout = din + in_bytes;
        cuda_check(copy_plane(din, plan.source_size * 4, input, is * 4, plan.source_size * 4,
                                     rows, cudaMemcpyHostToDevice, ws.stream), "uploading rows");
        PlaneTask t;
        t.horizontal = &plan;
        t.horizontal_keep = keep;
        t.input = din;
        t.input_stride = plan.source_size;
        t.output = dout;
        t.output_stride = plan.destination_size;
        t.vectors = rows;
        impl_->enqueue(ws, {t});
        cuda_check(copy_plane(output, os * 4, dout, plan.destination_size * 4,
                                     plan.destination_size * 4, rows, cudaMemcpyDeviceToHost, ws.stream),
                   "downloading rows");
        impl_->finish(ws);
    } catch (...) {
        cudaStreamSynchronize(ws.stream);
        impl_->release_slot(slot);
        throw;
    }
    impl_->release_slot(slot);
}

void Executor::inverse_columns(const AxisPlan &plan, const float *input, std::ptrdiff_t is,
                               float *output, std::ptrdiff_t os, std::int32_t columns,
                               const std::shared_ptr<const AxisPlan> &keep) {
    check_columns(plan, input, is, output, os, columns);
    if (columns == 0) return;
    DeviceGuard guard(impl_->device);
    std::size_t slot = 0;
    Workspace &ws = impl_->acquire_slot(slot);
    try {
        const std::size_t in_bytes = align_up(static_cast<std::size_t>(plan.source_size) * columns * 4);
        const std::size_t out_bytes = align_up(static_cast<std::size_t>(plan.destination_size) * columns * 4);
        ws.staging.reserve(in_bytes + out_bytes);
        char *din = ws.staging.data();
        char *dout = din + in_bytes;
        cuda_check(copy_plane(din, columns * 4, input, is * 4, columns * 4, plan.source_size,
                                     cudaMemcpyHostToDevice, ws.stream), "uploading columns");
        PlaneTask t;
        t.vertical = &plan;
        t.vertical_keep = keep;
        t.input = din;
        t.input_stride = columns;
        t.output = dout;
        t.output_stride = columns;
        t.vectors = columns;
        impl_->enqueue(ws, {t});
        cuda_check(copy_plane(output, os * 4, dout, columns * 4, columns * 4,
                                     plan.destination_size, cudaMemcpyDeviceToHost, ws.stream),
                   "downloading columns");
        impl_->finish(ws);
    } catch (...) {
        cudaStreamSynchronize(ws.stream);
        impl_->release_slot(slot);
        throw;
    }
    impl_->release_slot(slot);
}

namespace {

void check_2d(const AxisPlan &h, const AxisPlan &v, dev::Sample sample, const void *input, std::ptrdiff_t is,
              const void *output, std::ptrdiff_t os, const IntegerConversion &conv) {
    if (!h.valid() || !v.valid() || !input || !output || is < h.source_size
        || os < h.destination_size || sample == dev::Sample::f64)
        throw std::invalid_argument("invalid 2D executor arguments");
    if (sample != dev::Sample::f32) {
        const std::uint32_t limit = sample == dev::Sample::u8 ? 255U : 65535U;
        if (!(conv.input_scale > 0.0F) || !(conv.output_scale > 0.0F)
            || !std::isfinite(conv.input_offset) || !std::isfinite(conv.input_scale)
            || !std::isfinite(conv.output_scale) || !std::isfinite(conv.output_offset)
            || conv.output_maximum == 0U || conv.output_maximum > limit)
            throw std::invalid_argument("invalid integer 2D executor arguments");
    }
}

} // namespace

void Executor::inverse_2d_planes(const std::vector<HostPlane> &planes, std::size_t group_bytes) {
    for (const auto &p : planes) {
        if (!p.horizontal || !p.vertical) throw std::invalid_argument("host plane without plans");
        check_2d(*p.horizontal, *p.vertical, p.sample, p.input, p.input_stride, p.output, p.output_stride,
                 p.conversion);
    }
    if (planes.empty()) return;
    if (group_bytes == 0) group_bytes = impl_->pipe_group_bytes;
    auto in_row = [](const HostPlane &p) { return static_cast<std::size_t>(p.horizontal->source_size) * sample_bytes(p.sample); };
    auto out_row = [](const HostPlane &p) { return static_cast<std::size_t>(p.horizontal->destination_size) * sample_bytes(p.sample); };
    auto in_bytes = [&](const HostPlane &p) { return in_row(p) * static_cast<std::size_t>(p.vertical->source_size); };
    auto out_bytes = [&](const HostPlane &p) {
        return out_row(p) * static_cast<std::size_t>(p.vertical->destination_size);
    };
    auto pack = [](std::size_t v) { return (v + 15) / 16 * 16; };
    auto plane_bytes = [&](const HostPlane &p) { return pack(in_bytes(p)) + pack(out_bytes(p)); };
    // Groups of consecutive planes.  Group boundaries sit at byte positions
    // of the whole job: the first three groups grow (1/8, 1/4, 1/2 of
    // group_bytes) and the last three shrink alike, so that the first upload
    // and the last download, which nothing overlaps, stay short; the middle
    // is cut into equal parts of at most group_bytes.  Jobs under twice the
    // ramp split into four parts (1/6, 1/3, 1/3, 1/6).  A plane belongs to the
    // part holding its middle byte; empty parts vanish.
    std::size_t total = 0;
    for (const auto &p : planes) total += plane_bytes(p);
    std::vector<std::size_t> bounds;
    const std::size_t up[3] = {group_bytes / 8, group_bytes / 8 + group_bytes / 4,
                               group_bytes / 8 + group_bytes / 4 + group_bytes / 2};
    if (total <= 2 * up[2]) {
        bounds = {total / 6, total / 2, total - total / 6};
    } else {
        const std::size_t m0 = up[2], m1 = total - up[2];
        const std::size_t parts = std::max<std::size_t>(1, (m1 - m0 + group_bytes - 1) / group_bytes);
        bounds.assign(up, up + 3);
        for (std::size_t k = 1; k < parts; ++k) bounds.push_back(m0 + (m1 - m0) * k / parts);
        for (int k = 2; k >= 0; --k) bounds.push_back(total - up[k]);
    }
    std::vector<std::pair<std::size_t, std::size_t>> groups;   // [first, last)
    std::size_t most = 0;
    {
        std::size_t pos = 0, bi = 0, first = 0, bytes = 0;
        for (std::size_t i = 0; i < planes.size(); ++i) {
            const std::size_t pb = plane_bytes(planes[i]);
            while (bi < bounds.size() && pos + pb / 2 >= bounds[bi]) {
                if (i > first) {
                    groups.emplace_back(first, i);
                    most = std::max(most, bytes);
                }
                first = i;
                bytes = 0;
                ++bi;
            }
            bytes += pb;
            pos += pb;
        }
        groups.emplace_back(first, planes.size());
        most = std::max(most, bytes);
    }
    DeviceGuard guard(impl_->device);
    std::scoped_lock pipe_lock(impl_->pipe_mutex);
    for (auto &ws : impl_->pipe) {
        if (!ws) ws = std::make_unique<Workspace>(nullptr);
        ws->staging.reserve(most + kAlign);
    }
    CopyLanes &lanes = impl_->pipe_copies;
    lanes.create();
    // A group's staging holds its inputs back to back, then its outputs back
    // to back, each at a 16-byte boundary.  Planes whose rows are contiguous
    // on the host and whose host buffers follow one another exactly (a frame
    // ring in one allocation) travel in one copy per direction.
    struct Run {
        char *host = nullptr, *dev = nullptr;
        std::size_t bytes = 0;
    };
    auto flush = [](Run &r, cudaMemcpyKind kind, cudaStream_t s, const char *what) {
        if (r.bytes == 0) return;
        const bool up = kind == cudaMemcpyHostToDevice;
        cuda_check(cudaMemcpyAsync(up ? static_cast<void *>(r.dev) : static_cast<void *>(r.host),
                                   up ? static_cast<const void *>(r.host) : static_cast<const void *>(r.dev),
                                   r.bytes, kind, s), what);
        r = Run{};
    };
    auto extend = [&](Run &r, const void *host, char *dev, std::size_t bytes, cudaMemcpyKind kind,
                      cudaStream_t s, const char *what) {
        char *h = static_cast<char *>(const_cast<void *>(host));
        if (r.bytes && (r.host + r.bytes != h || r.dev + r.bytes != dev)) flush(r, kind, s, what);
        if (r.bytes == 0) {
            r.host = h;
            r.dev = dev;
        }
        r.bytes += bytes;
    };
    // Device addresses of page-locked host buffers (DSMVC_GB_HOST_DIRECT=1):
    // the kernels read such inputs and write such outputs in place.
    auto mapped = [&](const void *ptr) -> void * {
        if (!impl_->host_direct) return nullptr;
        cudaPointerAttributes a{};
        if (cudaPointerGetAttributes(&a, ptr) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
    };
    std::vector<void *> direct_in(planes.size()), direct_out(planes.size());
    for (std::size_t i = 0; i < planes.size(); ++i) {
        direct_in[i] = mapped(planes[i].input);
        direct_out[i] = mapped(planes[i].output);
    }
    std::size_t used = 0;
    try {
        for (std::size_t g = 0; g < groups.size(); ++g) {
            const std::size_t w = g % impl_->pipe.size();
            Workspace &ws = *impl_->pipe[w];
            used = std::max(used, w + 1);
            // The workspace's staging is free once its previous group's
            // downloads are done (which followed that group's kernels).
            if (g >= impl_->pipe.size())
                cuda_check(cudaStreamWaitEvent(lanes.up, lanes.downloaded[w], 0), "ordering uploads");
            std::size_t in_total = 0;
            for (std::size_t i = groups[g].first; i < groups[g].second; ++i)
                if (!direct_in[i]) in_total += pack(in_bytes(planes[i]));
            char *din = ws.staging.data();
            char *dout = din + in_total;
            std::vector<PlaneTask> tasks;
            std::vector<char *> outs;
            Run run;
            for (std::size_t i = groups[g].first; i < groups[g].second; ++i) {
                const HostPlane &p = planes[i];
                const std::size_t es = sample_bytes(p.sample);
                PlaneTask t;
                t.horizontal = p.horizontal;
                t.vertical = p.vertical;
                t.horizontal_keep = p.horizontal_keep;
                t.vertical_keep = p.vertical_keep;
                t.sample = p.sample;
                t.conversion = p.conversion;
                if (direct_in[i]) {
                    t.input = direct_in[i];
                    t.input_stride = p.input_stride;
                } else {
                    if (static_cast<std::size_t>(p.input_stride) * es == in_row(p)) {
                        extend(run, p.input, din, in_bytes(p), cudaMemcpyHostToDevice, lanes.up, "uploading planes");
                    } else {
                        flush(run, cudaMemcpyHostToDevice, lanes.up, "uploading planes");
                        cuda_check(copy_plane(din, in_row(p), p.input, p.input_stride * es, in_row(p),
                                              p.vertical->source_size, cudaMemcpyHostToDevice, lanes.up),
                                   "uploading plane");
                    }
                    t.input = din;
                    t.input_stride = p.horizontal->source_size;
                    din += pack(in_bytes(p));
                }
                if (direct_out[i]) {
                    t.output = direct_out[i];
                    t.output_stride = p.output_stride;
                    outs.push_back(nullptr);
                } else {
                    t.output = dout;
                    t.output_stride = p.horizontal->destination_size;
                    outs.push_back(dout);
                    dout += pack(out_bytes(p));
                }
                tasks.push_back(t);
            }
            flush(run, cudaMemcpyHostToDevice, lanes.up, "uploading planes");
            // The job table follows the planes on the upload stream (on the
            // workspace's stream it queued behind later groups' uploads).
            impl_->enqueue(ws, tasks, nullptr, 0, lanes.up);
            cuda_check(cudaEventRecord(lanes.computed[w], ws.stream), "recording event");
            cuda_check(cudaStreamWaitEvent(lanes.down, lanes.computed[w], 0), "ordering downloads");
            for (std::size_t i = groups[g].first, k = 0; i < groups[g].second; ++i, ++k) {
                if (!outs[k]) {
                    flush(run, cudaMemcpyDeviceToHost, lanes.down, "downloading planes");
                    continue;
                }
                const HostPlane &p = planes[i];
                const std::size_t es = sample_bytes(p.sample);
                if (static_cast<std::size_t>(p.output_stride) * es == out_row(p)) {
                    extend(run, p.output, outs[k], out_bytes(p), cudaMemcpyDeviceToHost, lanes.down,
                           "downloading planes");
                } else {
                    flush(run, cudaMemcpyDeviceToHost, lanes.down, "downloading planes");
                    cuda_check(copy_plane(p.output, p.output_stride * es, outs[k], out_row(p), out_row(p),
                                          p.vertical->destination_size, cudaMemcpyDeviceToHost, lanes.down),
                               "downloading plane");
                }
            }
            flush(run, cudaMemcpyDeviceToHost, lanes.down, "downloading planes");
            cuda_check(cudaEventRecord(lanes.downloaded[w], lanes.down), "recording event");
        }
        // Every group's downloads followed its kernels, which followed its
        // uploads: the download stream is the last to finish.
        cuda_check(cudaStreamSynchronize(lanes.down), "synchronizing");
        for (std::size_t k = 0; k < used; ++k) impl_->finish(*impl_->pipe[k]);
    } catch (...) {
        lanes.synchronize();
        for (std::size_t k = 0; k < used; ++k) cudaStreamSynchronize(impl_->pipe[k]->stream);
        throw;
    }
}

void Executor::inverse_2d(const AxisPlan &h, const AxisPlan &v, dev::Sample sample,
                          const void *input, std::ptrdiff_t is, void *output, std::ptrdiff_t os,
                          const IntegerConversion &conv, const std::shared_ptr<const AxisPlan> &h_keep,
                          const std::shared_ptr<const AxisPlan> &v_keep) {
    check_2d(h, v, sample, input, is, output, os, conv);
    const std::size_t es = sample_bytes(sample);
    DeviceGuard guard(impl_->device);
    std::size_t slot = 0;
    Workspace &ws = impl_->acquire_slot(slot);
    try {
        const std::size_t in_row = static_cast<std::size_t>(h.source_size) * es;
        const std::size_t out_row = static_cast<std::size_t>(h.destination_size) * es;
        const std::size_t in_bytes = align_up(in_row * v.source_size);
        const std::size_t out_bytes = align_up(out_row * v.destination_size);
        ws.staging.reserve(in_bytes + out_bytes);
        char *din = ws.staging.data();
        char *dout = din + in_bytes;
        cuda_check(copy_plane(din, in_row, input, is * es, in_row, v.source_size,
                                     cudaMemcpyHostToDevice, ws.stream), "uploading plane");
        PlaneTask t;
        t.horizontal = &h;
        t.vertical = &v;
        t.horizontal_keep = h_keep;
        t.vertical_keep = v_keep;
        t.input = din;
        t.input_stride = h.source_size;
        t.output = dout;
        t.output_stride = h.destination_size;
        t.sample = sample;
        t.conversion = conv;
        impl_->enqueue(ws, {t});
        cuda_check(copy_plane(output, os * es, dout, out_row, out_row, v.destination_size,
                                     cudaMemcpyDeviceToHost, ws.stream), "downloading plane");
        impl_->finish(ws);
    } catch (...) {
        cudaStreamSynchronize(ws.stream);
        impl_->release_slot(slot);
        throw;
    }
    impl_->release_slot(slot);
}

namespace {

void validate_tasks(const std::vector<PlaneTask> &tasks) {
    for (const auto &t : tasks) {
        const AxisPlan *h = t.horizontal, *v = t.vertical;
        if ((!h && !v) || !t.input || (!t.output && !t.score) || (h && !h->valid()) || (v && !v->valid()))
            throw std::invalid_argument("invalid batch plane");
        if (t.score && (!h || !v || t.sample != dev::Sample::f32 || t.score_tiles <= 0))
            throw std::invalid_argument("invalid fused scoring task");
        if (h && v) {
            if (t.input_stride < h->source_size || t.output_stride < h->destination_size)
                throw std::invalid_argument("invalid batch plane strides");
        } else if (h) {
            if (t.sample != dev::Sample::f32 || t.vectors < 0 || t.input_stride < h->source_size
                || t.output_stride < h->destination_size)
                throw std::invalid_argument("invalid batch row task");
        } else {
            if (t.sample != dev::Sample::f32 || t.vectors < 0 || t.input_stride < t.vectors
                || t.output_stride < t.vectors)
                throw std::invalid_argument("invalid batch column task");
        }
    }
}

} // namespace

void Executor::run_batch(const std::vector<PlaneTask> &tasks, void *stream, bool synchronize, void *scratch,
                         std::size_t scratch_capacity) {
    DeviceGuard guard(impl_->device);
    validate_tasks(tasks);
    Workspace &ws = impl_->stream_space(static_cast<cudaStream_t>(stream));
    impl_->enqueue(ws, tasks, static_cast<char *>(scratch), scratch_capacity);
    if (synchronize) impl_->finish(ws);
}

struct PreparedBatch::Impl {
    Executor::Impl *owner = nullptr;
    // The tasks in one part, or two (each half of the work) whose launches
    // run on two streams forked from the caller's and joined back to it.
    struct Part {
        Executor::Impl::Compiled compiled;
        DeviceBuffer scratch;             // unused with caller-owned scratch
        DeviceBuffer table;
    };
    std::vector<std::unique_ptr<Part>> parts;
    cudaStream_t side = nullptr;           // the second part's stream
    cudaEvent_t fork = nullptr, join = nullptr;
    std::uint32_t *status = nullptr;       // device
    std::uint32_t *status_host = nullptr;  // pinned
    ~Impl() {
        if (join) cudaEventDestroy(join);
        if (fork) cudaEventDestroy(fork);
        if (side) cudaStreamDestroy(side);
        if (status) cudaFree(status);
        if (status_host) cudaFreeHost(status_host);
    }
    // Launch group `index` counted across the parts.
    std::pair<const Part *, std::size_t> group(std::size_t index) const {
        for (const auto &pt : parts) {
            if (index < pt->compiled.launches.size()) return {pt.get(), index};
            index -= pt->compiled.launches.size();
        }
        throw std::out_of_range("launch group index");
    }
};

PreparedBatch::PreparedBatch(std::unique_ptr<Impl> impl) : impl_(std::move(impl)) {}

PreparedBatch::~PreparedBatch() {
    if (!impl_) return;
    DeviceGuard guard(impl_->owner->device);
    // Kernels of an earlier launch may still read the table and scratch.
    cudaDeviceSynchronize();
    impl_.reset();
}

void PreparedBatch::launch(void *stream) {
    DeviceGuard guard(impl_->owner->device);
    auto s = static_cast<cudaStream_t>(stream);
    auto &m = *impl_;
    if (m.parts.size() == 1) {
        m.owner->launch(m.parts[0]->compiled, m.parts[0]->table.data(), s, m.status);
        return;
    }
    // Fork: the second part's stream waits for the caller's; join: the
    // caller's waits for it.  Both are stream-ordered (capturable).
    cuda_check(cudaEventRecord(m.fork, s), "recording fork");
    cuda_check(cudaStreamWaitEvent(m.side, m.fork, 0), "forking");
    m.owner->launch(m.parts[0]->compiled, m.parts[0]->table.data(), s, m.status);
    m.owner->launch(m.parts[1]->compiled, m.parts[1]->table.data(), m.side, m.status);
    cuda_check(cudaEventRecord(m.join, m.side), "recording join");
    cuda_check(cudaStreamWaitEvent(s, m.join, 0), "joining");
}

void PreparedBatch::launch_group(std::size_t index, void *stream) {
    DeviceGuard guard(impl_->owner->device);
    const auto [part, i] = impl_->group(index);
    Executor::Impl::Compiled one;
    one.launches.push_back(part->compiled.launches[i]);
    impl_->owner->launch(one, part->table.data(), static_cast<cudaStream_t>(stream), impl_->status);
}

std::vector<BatchGroup> PreparedBatch::groups() const {
    std::vector<BatchGroup> out;
    for (const auto &pt : impl_->parts)
    for (const auto &l : pt->compiled.launches) {
        BatchGroup g;
        g.key = {l.pass, l.kind, l.hb, static_cast<int>(l.in), static_cast<int>(l.out), l.variant};
        g.kind = l.kind;
        g.threads = l.threads;
        g.blocks = l.blocks;
        g.jobs = l.count;
        g.name = kernel_name({l.pass, l.kind, l.hb, l.in, l.out, l.variant});
        out.push_back(g);
    }
    return out;
}

void PreparedBatch::check_status(void *stream) {
    DeviceGuard guard(impl_->owner->device);
    auto s = static_cast<cudaStream_t>(stream);
    cuda_check(cudaMemcpyAsync(impl_->status_host, impl_->status, sizeof(std::uint32_t),
                               cudaMemcpyDeviceToHost, s), "reading status");
    cuda_check(cudaStreamSynchronize(s), "synchronizing");
    const std::uint32_t status = *impl_->status_host;
    if (status) {
        cuda_check(cudaMemset(impl_->status, 0, sizeof(std::uint32_t)), "clearing status");
        throw_status(status);
    }
}

std::size_t PreparedBatch::kernel_launches() const {
    std::size_t n = 0;
    for (const auto &pt : impl_->parts) n += pt->compiled.launches.size();
    return n;
}
std::size_t PreparedBatch::scratch_bytes() const {
    std::size_t n = 0;
    for (const auto &pt : impl_->parts) n += pt->compiled.scratch_bytes;
    return n;
}
std::size_t PreparedBatch::table_bytes() const {
    std::size_t n = 0;
    for (const auto &pt : impl_->parts) n += pt->compiled.table.size();
    return n;
}
std::size_t PreparedBatch::parts() const { return impl_->parts.size(); }

std::size_t Executor::batch_scratch_bound(const std::vector<PlaneTask> &tasks) {
    // Per task: the intermediate plane (destinations of the first pass x
    // sources of the second, rows padded to 4) plus a forward plane of the
    // output's size, in the route's sample width; 2D planes also the forward
    // values of two-pass segments (margins included, at most twice a pass's
    // whole chunks of forward values).  A fused scoring task's columns pass
    // needs nothing beyond the intermediate.
    std::size_t bytes = kAlign;
    for (const auto &t : tasks) {
        const AxisPlan *h = t.horizontal, *v = t.vertical;
        if (!h && !v) continue;
        const bool f64 = (h && h->requires_float64()) || (v && v->requires_float64());
        const std::size_t es = f64 ? 8 : 4;
        const std::size_t hd = h ? static_cast<std::size_t>(h->destination_size) : static_cast<std::size_t>(t.vectors);
        const std::size_t vs = v ? (static_cast<std::size_t>(v->source_size) + 3) / 4 * 4 : static_cast<std::size_t>(t.vectors);
        const std::size_t vd = v ? static_cast<std::size_t>(v->destination_size) : static_cast<std::size_t>(t.vectors);
        bytes += align_up(hd * vs * es) + (t.score ? 0 : align_up(hd * vd * es));
        if (h && v) {
            const std::size_t hc = (hd + kStreamChunk - 1) / kStreamChunk * kStreamChunk;
            const std::size_t vc = (vd + kStreamChunk - 1) / kStreamChunk * kStreamChunk;
            bytes += align_up(2 * hc * vs * es) + (t.score ? 0 : align_up(2 * vc * hd * es));
        }
    }
    return bytes;
}

int Executor::fused_scoring_window(const AxisPlan &vertical, const std::shared_ptr<const AxisPlan> &keep) {
    DeviceGuard guard(impl_->device);
    if (!vertical.valid()) throw std::invalid_argument("invalid plan");
    if (vertical.requires_float64()) return -1;
    std::vector<std::shared_ptr<DevicePlan>> held;
    int private_uploads = 0;
    return impl_->fused_window(impl_->device_plan(vertical, keep, held, private_uploads));
}

std::unique_ptr<PreparedBatch> Executor::prepare_batch(const std::vector<PlaneTask> &tasks,
                                                       const BatchTuning *tuning, void *scratch,
                                                       std::size_t scratch_capacity, int vectors_per_warp,
                                                       int parts) {
    DeviceGuard guard(impl_->device);
    validate_tasks(tasks);
    if (vectors_per_warp != 0 && vectors_per_warp != 32 && vectors_per_warp != 64)
        throw std::invalid_argument("vectors per warp must be 0, 32 or 64");
    for (const auto &[key, threads] : tuning ? *tuning : BatchTuning{}) {
        const int kind = key[1];
        const int most = kind >= 3 && kind <= 6 ? 256 : 128;
        if (kind == 2 || kind > 6 || threads < 32 || threads > most || threads % 32)
            throw std::invalid_argument("invalid CTA size in batch tuning");
    }
    Executor::Impl::Tuning t;
    if (tuning)
        for (const auto &[k, v] : *tuning) t[{k[0], k[1], k[2], k[3], k[4], k[5]}] = v;
    auto b = std::make_unique<PreparedBatch::Impl>();
    b->owner = impl_.get();
    cuda_check(cudaMalloc(&b->status, sizeof(std::uint32_t)), "allocating status");
    cuda_check(cudaMallocHost(&b->status_host, sizeof(std::uint32_t)), "allocating status");
    cuda_check(cudaMemset(b->status, 0, sizeof(std::uint32_t)), "clearing status");
    // Two parts (launches overlapping on two streams: one part's second pass
    // runs beside the other's first) for batches of many tasks that own
    // their scratch; split where the source pixels are halved.
    int n_parts = parts;
    if (n_parts == 0) n_parts = !scratch && tasks.size() >= kSplitBatchTasks ? 2 : 1;
    if (n_parts != 1 && n_parts != 2) throw std::invalid_argument("a prepared batch has 1 or 2 parts");
    if (n_parts == 2 && (scratch || tasks.size() < 2))
        throw std::invalid_argument("two batch parts need two tasks and batch-owned scratch");
    std::size_t cut = tasks.size();
    if (n_parts == 2) {
        auto work = [](const PlaneTask &t) {
            const auto rows = t.vertical ? t.vertical->source_size : t.vectors;
            const auto cols = t.horizontal ? t.horizontal->source_size : t.vectors;
            return static_cast<double>(rows) * static_cast<double>(cols);
        };
        double total = 0.0, acc = 0.0;
        for (const auto &t : tasks) total += work(t);
        cut = 1;
        for (std::size_t i = 0; i + 1 < tasks.size(); ++i) {
            acc += work(tasks[i]);
            cut = i + 1;
            if (acc >= total / 2) break;
        }
    }
    for (int k = 0; k < n_parts; ++k) {
        b->parts.push_back(std::make_unique<PreparedBatch::Impl::Part>());
        auto &pt = *b->parts.back();
        const std::vector<PlaneTask> part_tasks = n_parts == 1 ? tasks
            : k == 0 ? std::vector<PlaneTask>(tasks.begin(), tasks.begin() + static_cast<std::ptrdiff_t>(cut))
                     : std::vector<PlaneTask>(tasks.begin() + static_cast<std::ptrdiff_t>(cut), tasks.end());
        impl_->compile(part_tasks, pt.compiled, [&](std::size_t bytes) {
            if (scratch) {
                if (bytes > scratch_capacity) throw std::length_error("batch scratch exceeds the caller's buffer");
                return static_cast<char *>(scratch);
            }
            pt.scratch.reserve(bytes);
            return pt.scratch.data();
        }, b->status, &t, vectors_per_warp);
        const auto &table = pt.compiled.table;
        pt.table.reserve(std::max<std::size_t>(table.size(), 1));
        if (!table.empty())
            cuda_check(cudaMemcpy(pt.table.data(), table.data(), table.size(), cudaMemcpyHostToDevice),
                       "uploading job table");
    }
    if (n_parts == 2) {
        cuda_check(cudaStreamCreateWithFlags(&b->side, cudaStreamNonBlocking), "creating stream");
        cuda_check(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming), "creating event");
        cuda_check(cudaEventCreateWithFlags(&b->join, cudaEventDisableTiming), "creating event");
    }
    return std::make_unique<PreparedBatch>(std::move(b));
}

void Executor::release_stream(void *stream) {
    DeviceGuard guard(impl_->device);
    std::unique_ptr<Workspace> ws;
    {
        std::scoped_lock lock(impl_->mutex);
        auto it = impl_->stream_spaces.find(static_cast<cudaStream_t>(stream));
        if (it == impl_->stream_spaces.end()) return;
        ws = std::move(it->second);
        impl_->stream_spaces.erase(it);
    }
    cuda_check(cudaStreamSynchronize(static_cast<cudaStream_t>(stream)), "synchronizing");
}

void Executor::check_status(void *stream) {
    DeviceGuard guard(impl_->device);
    impl_->finish(impl_->stream_space(static_cast<cudaStream_t>(stream)));
}

void Executor::set_profiling(bool enable) {
    DeviceGuard guard(impl_->device);
    std::scoped_lock lock(impl_->mutex);
    impl_->records.clear();
    impl_->events_used = 0;
    impl_->profiling = enable;
}

std::vector<KernelTime> Executor::kernel_times() {
    DeviceGuard guard(impl_->device);
    std::scoped_lock lock(impl_->mutex);
    std::vector<KernelTime> out;
    for (auto &r : impl_->records) {
        cuda_check(cudaEventSynchronize(r.stop), "waiting for profiled kernel");
        float ms = 0.0F;
        cuda_check(cudaEventElapsedTime(&ms, r.start, r.stop), "reading event");
        auto it = std::find_if(out.begin(), out.end(), [&](const KernelTime &k) { return k.name == r.name; });
        if (it == out.end()) {
            out.push_back({r.name, 0, 0.0, 0});
            it = out.end() - 1;
        }
        it->launches += 1;
        it->milliseconds += ms;
        it->bytes += r.bytes;
    }
    return out;
}

ExecutorStats Executor::stats() const {
    std::scoped_lock lock(impl_->mutex);
    ExecutorStats s = impl_->stats;
    s.plan_cache_bytes = impl_->cache_bytes;
    for (const auto &ws : impl_->slots) s.workspace_bytes += ws->scratch.size() + ws->staging.size();
    for (const auto &[k, ws] : impl_->stream_spaces) s.workspace_bytes += ws->scratch.size();
    return s;
}

} // namespace dsmvc_gb
