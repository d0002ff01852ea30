// Device-side data structures shared by the descale kernels and the host
// executor.  Plain PODs: they cross the host/device boundary by value or in
// device job tables.
#pragma once

#include <cstdint>

namespace dsmvc_gb::dev {

// One uploaded axis plan (see executor.cpp: DevicePlan).  Every pointer is
// into a single device allocation.  Band arrays follow the reference plan
// layout (include/dsmvc/engine.hpp:82-138): lower[(d-1)*n+i], upper[(d-1)*n+i],
// bands64[d*n+i] with band 0 holding D.
struct PlanView {
    std::int32_t source_size;
    std::int32_t destination_size;
    std::int32_t half_bandwidth;
    std::int32_t retains_f64;   // 1: use weights64/bands64 in the F64 route
    const std::uint32_t *offsets;
    const std::int32_t *indices;
    const float *weights;
    const float *lower;
    const float *upper;
    const float *inv_diag;
    const double *weights64;
    const double *bands64;
    const double *normal64;     // unfactored normal band G (Float64 plans), band d at d*n+i
};

// IntegerConversion (include/dsmvc/engine.hpp:167-173).
struct Conversion {
    float in_offset;
    float in_scale;
    float out_scale;
    float out_offset;
    std::uint32_t out_max;
};

// One batch of independent vectors solved with one plan.  Element k of
// vector v of an array X lives at X + k * X_elem + v * X_vec (in samples).
// `fwd` receives the forward-substitution values, read back by the backward
// pass; it may alias `out` when `out` is a float array of the same layout.
struct AxisJob {
    PlanView plan;
    const void *in;
    std::int64_t in_elem, in_vec;
    void *out;
    std::int64_t out_elem, out_vec;
    void *fwd;
    std::int64_t fwd_elem, fwd_vec;
    std::int32_t vectors;
    std::int32_t first_block;   // exclusive prefix sum of blocks per job
    Conversion conv;
};

// Status bits written by kernels (read back by the executor).
enum StatusBits : std::uint32_t {
    kStatusNonFiniteInput = 1U,
    kStatusNonFiniteOutput = 2U,
    kStatusFeedStall = 4U,         // a streaming kernel's staged feed wait ran out
};

enum class Sample : std::int32_t { f32 = 0, u8 = 1, u16 = 2, f64 = 3 };

} // namespace dsmvc_gb::dev

namespace dsmvc_gb {

// Kernel launchers (kernels.cu).  `jobs` is a device array; every job of one
// launch has the same half-bandwidth, input and output sample kinds.
// Returns cudaError_t as int.
int launch_axis_f32(const dev::AxisJob *jobs, int job_count, int total_blocks,
                    int threads, int half_bandwidth, dev::Sample in,
                    dev::Sample out, void *stream);
int launch_axis_f64(const dev::AxisJob *jobs, int job_count, int total_blocks,
                    int threads, int half_bandwidth, dev::Sample in,
                    dev::Sample out, std::uint32_t *status, void *stream);
// Float64 residual refinement of solved vectors and the conversion of a
// Float64 result (refine64.cu); 32..128 threads a block, one vector (or
// output row) per thread.
int launch_refine64(const dev::AxisJob *jobs, int job_count, int total_blocks,
                    int threads, int half_bandwidth, dev::Sample in,
                    std::uint32_t *status, void *stream);
int launch_convert64(const dev::AxisJob *jobs, int job_count, int total_blocks,
                     int threads, dev::Sample out, std::uint32_t *status, void *stream);

} // namespace dsmvc_gb
