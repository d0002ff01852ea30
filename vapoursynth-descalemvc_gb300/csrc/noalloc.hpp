// Allocation-free 2D descale (noalloc.cu).
#pragma once

#include "kernels.cuh"
#include "planner.hpp"

#include <cstddef>
#include <cstdint>

namespace dsmvc_gb {

// Size of the file-scope device array the entry point works in: the job
// table, both plans' coefficients, the Float32 intermediate plane
// (4 bytes x vertical source size x horizontal destination size) and, for
// integer output, a forward scratch plane of the output's size.
constexpr std::size_t kNoAllocBytes = std::size_t{32} << 20;

// Enqueues the Float32 2D descale of `input` into `output` (device pointers,
// strides in samples) on `stream` without allocating.  The plan uploads come
// from pageable host memory, so the call may block the host until they are
// done.  Throws std::invalid_argument for Float64 plans, for frames that do
// not fit kNoAllocBytes and for a stream that is being captured.
void inverse_2d_noalloc(const AxisPlan &horizontal, const AxisPlan &vertical, dev::Sample sample,
                        const void *input, std::int64_t input_stride, void *output,
                        std::int64_t output_stride, const dev::Conversion &conversion,
                        void *stream);

} // namespace dsmvc_gb
