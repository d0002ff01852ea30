// Allocation-free 2D descale: the Float32 route of the 2D descale (the
// sequential axis kernels of kernels.cu, rows then columns) for callers that
// must not allocate device memory, e.g. code running inside another
// framework's memory pool or allocator-free real-time pipelines.
//
// Everything the kernels need besides the caller's input and output -- the
// two-entry job table, both plans' coefficients and the Float32 intermediate
// plane (plus a forward scratch plane for integer output) -- lives in one
// file-scope __device__ array of kNoAllocBytes.  Every GPU that loads this
// library holds that array until the process exits.  The host reaches it
// through cudaGetSymbolAddress, once per device on the device's first call;
// in host code the array's name is only a stand-in, never a device address.
// The looked-up address is kept for the life of the process, so the entry
// point must not be used on a device after cudaDeviceReset.
//
// Each call copies the job table and both plans' coefficients into the
// array from pageable host memory (the plans' own vectors and a job table on
// the caller's stack) with cudaMemcpyAsync: the call may block the host
// until those copies are done, and it refuses a stream that is being
// captured, whose copies would point at host memory gone by the time the
// work runs.  All calls share the array, so calls whose work overlaps on the
// GPU (different streams, or the same stream from several threads without
// ordering) race on it.  No part of it needs to start at zero: every byte a
// call reads was written earlier by the same call.
#include "noalloc.hpp"

#include "kernels.cuh"

#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <mutex>
#include <stdexcept>
#include <string>

namespace dsmvc_gb {
namespace {

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

constexpr int kMaxDevices = 64;
constexpr int kThreads = 128;
constexpr std::size_t kAlign = 256;

std::mutex g_mutex;
void *g_address[kMaxDevices] = {};

std::size_t align_up(std::size_t v) { return (v + kAlign - 1) / kAlign * kAlign; }

void check(cudaError_t e, const char *what) {
    if (e != cudaSuccess)
        throw std::runtime_error(std::string("CUDA ") + what + ": " + cudaGetErrorString(e));
}

// Device address of the scratch array on the current device.
char *scratch_address() {
    int device = -1;
    check(cudaGetDevice(&device), "querying the device");
    if (device < 0 || device >= kMaxDevices)
        throw std::runtime_error("device ordinal beyond the allocation-free entry point's table");
    std::scoped_lock lock(g_mutex);
    if (!g_address[device]) {
        void *p = nullptr;
        check(cudaGetSymbolAddress(&p, g_noalloc_scratch), "locating the scratch array");
        g_address[device] = p;
    }
    return static_cast<char *>(g_address[device]);
}

// Byte layout of one plan's arrays inside the scratch array.
struct PlanLayout {
    std::size_t offsets, indices, weights, lower, upper, inv_diag, end;
};

PlanLayout layout_of(const AxisPlan &p, std::size_t at) {
    PlanLayout l{};
    l.offsets = at;
    l.indices = align_up(l.offsets + p.transpose_offsets.size() * 4);
    l.weights = align_up(l.indices + p.transpose_indices.size() * 4);
    l.lower = align_up(l.weights + p.transpose_weights.size() * 4);
    l.upper = align_up(l.lower + p.lower_ld.size() * 4);
    l.inv_diag = align_up(l.upper + p.upper_l.size() * 4);
    l.end = align_up(l.inv_diag + p.inverse_diagonal.size() * 4);
    return l;
}

template <class T>
void copy_array(char *base, std::size_t at, const std::vector<T> &v, cudaStream_t s) {
    if (v.empty()) return;
    check(cudaMemcpyAsync(base + at, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s),
          "copying plan coefficients");
}

dev::PlanView view_of(const AxisPlan &p, const PlanLayout &l, char *base) {
    dev::PlanView v{};
    v.source_size = p.source_size;
    v.destination_size = p.destination_size;
    v.half_bandwidth = p.half_bandwidth;
    v.retains_f64 = 0;
    v.offsets = reinterpret_cast<const std::uint32_t *>(base + l.offsets);
    v.indices = reinterpret_cast<const std::int32_t *>(base + l.indices);
    v.weights = reinterpret_cast<const float *>(base + l.weights);
    v.lower = reinterpret_cast<const float *>(base + l.lower);
    v.upper = reinterpret_cast<const float *>(base + l.upper);
    v.inv_diag = reinterpret_cast<const float *>(base + l.inv_diag);
    return v;
}

} // namespace

void inverse_2d_noalloc(const AxisPlan &h, const AxisPlan &v, dev::Sample sample,
                        const void *input, std::int64_t input_stride, void *output,
                        std::int64_t output_stride, const dev::Conversion &conv, void *stream) {
    if (!h.valid() || !v.valid() || !input || !output || input_stride < h.source_size
        || output_stride < h.destination_size
        || (sample != dev::Sample::f32 && sample != dev::Sample::u8 && sample != dev::Sample::u16))
        throw std::invalid_argument("invalid allocation-free 2D arguments");
    if (h.requires_float64() || v.requires_float64())
        throw std::invalid_argument(
            "the allocation-free entry point runs the Float32 route only; this plan needs Float64");
    if (sample != dev::Sample::f32) {
        const std::uint32_t limit = sample == dev::Sample::u8 ? 255U : 65535U;
        if (!(conv.in_scale > 0.0F) || !(conv.out_scale > 0.0F) || !std::isfinite(conv.in_offset)
            || !std::isfinite(conv.in_scale) || !std::isfinite(conv.out_scale)
            || !std::isfinite(conv.out_offset) || conv.out_max == 0U || conv.out_max > limit)
            throw std::invalid_argument("invalid integer conversion");
    }
    // Layout: job table, both plans, the intermediate, then (integer output)
    // a forward scratch plane.
    const std::size_t jobs_at = 0;
    const PlanLayout lh = layout_of(h, align_up(2 * sizeof(dev::AxisJob)));
    const PlanLayout lv = layout_of(v, lh.end);
    const std::size_t mid_stride = static_cast<std::size_t>(h.destination_size);
    const std::size_t mid_at = lv.end;
    const std::size_t fwd_at = align_up(mid_at + mid_stride * static_cast<std::size_t>(v.source_size) * 4);
    const std::size_t end = sample == dev::Sample::f32
        ? fwd_at : align_up(fwd_at + mid_stride * static_cast<std::size_t>(v.destination_size) * 4);
    if (end > kNoAllocBytes)
        throw std::invalid_argument("frame needs " + std::to_string(end) + " bytes of scratch; the "
                                    "allocation-free entry point holds " + std::to_string(kNoAllocBytes));

    auto s = static_cast<cudaStream_t>(stream);
    cudaStreamCaptureStatus capture = cudaStreamCaptureStatusNone;
    check(cudaStreamIsCapturing(s, &capture), "querying the stream's capture status");
    if (capture != cudaStreamCaptureStatusNone)
        throw std::invalid_argument("the allocation-free entry point copies its plans from pageable "
                                    "host memory and cannot run on a stream that is being captured");
    char *base = scratch_address();
    copy_array(base, lh.offsets, h.transpose_offsets, s);
    copy_array(base, lh.indices, h.transpose_indices, s);
    copy_array(base, lh.weights, h.transpose_weights, s);
    copy_array(base, lh.lower, h.lower_ld, s);
    copy_array(base, lh.upper, h.upper_l, s);
    copy_array(base, lh.inv_diag, h.inverse_diagonal, s);
    copy_array(base, lv.offsets, v.transpose_offsets, s);
    copy_array(base, lv.indices, v.transpose_indices, s);
    copy_array(base, lv.weights, v.transpose_weights, s);
    copy_array(base, lv.lower, v.lower_ld, s);
    copy_array(base, lv.upper, v.upper_l, s);
    copy_array(base, lv.inv_diag, v.inverse_diagonal, s);

    dev::AxisJob jobs[2] = {};
    float *mid = reinterpret_cast<float *>(base + mid_at);
    auto &row = jobs[0];
    row.plan = view_of(h, lh, base);
    row.in = input;
    row.in_elem = 1;
    row.in_vec = input_stride;
    row.out = mid;
    row.out_elem = 1;
    row.out_vec = static_cast<std::int64_t>(mid_stride);
    row.fwd = mid;
    row.fwd_elem = 1;
    row.fwd_vec = row.out_vec;
    row.vectors = v.source_size;
    row.first_block = 0;
    row.conv = conv;
    auto &col = jobs[1];
    col.plan = view_of(v, lv, base);
    col.in = mid;
    col.in_elem = static_cast<std::int64_t>(mid_stride);
    col.in_vec = 1;
    col.out = output;
    col.out_elem = output_stride;
    col.out_vec = 1;
    if (sample == dev::Sample::f32) {
        col.fwd = output;
        col.fwd_elem = output_stride;
    } else {
        col.fwd = base + fwd_at;
        col.fwd_elem = static_cast<std::int64_t>(mid_stride);
    }
    col.fwd_vec = 1;
    col.vectors = h.destination_size;
    col.first_block = 0;
    col.conv = conv;
    check(cudaMemcpyAsync(base + jobs_at, jobs, sizeof(jobs), cudaMemcpyHostToDevice, s),
          "copying the job table");
    const auto *dev_jobs = reinterpret_cast<const dev::AxisJob *>(base + jobs_at);
    const int row_blocks = (row.vectors + kThreads - 1) / kThreads;
    const int col_blocks = (col.vectors + kThreads - 1) / kThreads;
    int rc = launch_axis_f32(dev_jobs, 1, row_blocks, kThreads, h.half_bandwidth, sample,
                             dev::Sample::f32, stream);
    check(static_cast<cudaError_t>(rc), "launching the row pass");
    rc = launch_axis_f32(dev_jobs + 1, 1, col_blocks, kThreads, v.half_bandwidth, dev::Sample::f32,
                         sample, stream);
    check(static_cast<cudaError_t>(rc), "launching the column pass");
}

} // namespace dsmvc_gb
