// Host planner for the GB300 descale executor: builds the inverse-only axis
// plan (CSR of A^T, banded LDL^T factor of A^T A, condition estimate) in
// FP64, exactly as the reference planner does, so that plans are
// bit-identical to the reference's (same FNV plan hashes).
//
// Types mirror include/dsmvc/engine.hpp:16-138 of the reference:
// KernelSpec, AxisRequest, AxisPlan, PlannerCacheStats.
#pragma once

#include <cstddef>
#include <cstdint>
#include <functional>
#include <memory>
#include <vector>

namespace dsmvc_gb {

enum class KernelKind : std::uint8_t {
    bilinear, bicubic, lanczos, spline16, spline36, spline64, custom,
};

enum class BorderMode : std::uint8_t {
    zero = 0, repeat = 1, reflect101 = 2, symmetric = 3, mirror = 4,
};

enum class F64Mode : std::uint8_t {
    automatic = 0, float32_only = 1, float64_only = 2,
};

struct KernelSpec {
    KernelKind kind = KernelKind::bicubic;
    std::int32_t taps = 3;
    double b = 0.0;
    double c = 0.5;
    double blur = 1.0;
};

struct AxisRequest {
    std::int32_t source_size = 0;
    std::int32_t destination_size = 0;
    double active_length = 0.0;
    double shift = 0.0;
    KernelSpec kernel{};
    BorderMode border = BorderMode::symmetric;
    F64Mode f64_mode = F64Mode::automatic;
};

using CustomKernel = std::function<double(double)>;

// Immutable plan.  Field meanings follow the reference AxisPlan
// (include/dsmvc/engine.hpp:82-138):
//   transpose_*        CSR of A^T, ascending source index per destination;
//   lower_ld[(d-1)n+i] L(i,i-d) * D(i-d), upper_l[(d-1)n+i] L(i+d,i);
//   inverse_diagonal   1 / (D + DBL_EPSILON) rounded to float;
//   *_f64              retained only when the plan needs Float64.
struct AxisPlan {
    std::int32_t source_size = 0;
    std::int32_t destination_size = 0;
    std::int32_t support = 0;
    std::int32_t half_bandwidth = 0;
    double active_length = 0.0;
    double shift = 0.0;

    std::vector<std::uint32_t> transpose_offsets;
    std::vector<std::int32_t> transpose_indices;
    std::vector<float> transpose_weights;
    std::vector<float> lower_ld;
    std::vector<float> upper_l;
    std::vector<float> inverse_diagonal;

    double normal_rcond = 1.0;
    double normal_inf_norm = 0.0;
    std::vector<double> transpose_weights_f64;
    std::vector<double> normal_bands_f64;
    std::vector<double> ldlt_bands_f64;
    std::vector<double> inverse_diagonal_f64;

    // Largest number of A^T entries in one destination row.
    std::int32_t max_row_entries = 0;
    // Set by build_axis_plan once the full check has passed: plans are
    // immutable afterwards, so valid() answers at once (executor calls check
    // every plan they are given).
    bool validated = false;

    [[nodiscard]] bool requires_float64() const noexcept {
        return !ldlt_bands_f64.empty();
    }
    [[nodiscard]] std::size_t storage_bytes() const noexcept;
    // Structural and finiteness checks of AxisPlan::check_valid
    // (src/axis_plan.cpp:1259-1341).
    [[nodiscard]] bool valid() const noexcept;
};

struct PlannerCacheStats {
    std::uint64_t plan_hits = 0;
    std::uint64_t plan_builds = 0;
    std::size_t plan_entries = 0;
    std::size_t plan_resident_bytes = 0;
};

// build_axis_plan (src/axis_plan.cpp:1351-1356).  Throws
// std::invalid_argument, std::length_error, std::out_of_range or
// std::runtime_error with the reference's conditions.
[[nodiscard]] AxisPlan build_axis_plan(const AxisRequest &request,
                                       const CustomKernel &custom = {});

// get_or_build_axis_plan (src/axis_plan.cpp:1358-1383): single-flight LRU
// keyed by the request (2048 entries / 256 MiB); custom kernels bypass it.
[[nodiscard]] std::shared_ptr<const AxisPlan> get_or_build_axis_plan(
    const AxisRequest &request, const CustomKernel &custom = {});

// Many plans at once with their normal band, banded LDL^T, condition
// estimate and Float32 arrays computed on the GPU `device` (-1: the current
// one), the geometry, kernel weights and A^T CSR on up to `threads` host
// threads (0: one per hardware thread).  Plans equal build_axis_plan's bit
// for bit (same plan hashes).  Custom kernels are refused (they plan on the
// host); the plan cache is not consulted.
[[nodiscard]] std::vector<AxisPlan> build_axis_plans_on_device(
    const std::vector<AxisRequest> &requests, int device, int threads);

[[nodiscard]] PlannerCacheStats planner_cache_stats();
void clear_planner_caches();

// FNV-1a hashes of tests/numerical_conformance.hpp:193-248 (conformance).
[[nodiscard]] std::uint64_t f32_plan_hash(const AxisRequest &request,
                                          const AxisPlan &plan);
[[nodiscard]] std::uint64_t complete_plan_hash(const AxisRequest &request,
                                               const AxisPlan &plan);

// detail::padding_index (src/axis_plan.cpp:1024-1066).
[[nodiscard]] std::int32_t padding_index(std::int64_t index,
                                         std::int32_t size, BorderMode mode);

} // namespace dsmvc_gb
