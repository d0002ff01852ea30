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
// strides in samples) on `stream` without allocating.  Throws
// std::invalid_argument for Float64 plans and for frames that do not fit
// kNoAllocBytes.
void inverse_2d_noalloc(const AxisPlan &horizontal, const AxisPlan &vertical, dev::Sample sample,
                        const void *input, std::int64_t input_stride, void *output,
                        std::int64_t output_stride, const dev::Conversion &conversion,
                        void *stream);

} // namespace dsmvc_gb
