// Drop-in CUDA backend for the reference engine: a class with the public
// interface of dsmvc::cuda_detail::CudaExecutor (src/cuda/cuda_executor.hpp:
// 11-110) whose work runs on the GB300 executor through its C ABI
// (include/dsmvc_gb300.h).  A maintainer swaps it in for CudaExecutor in the
// reference's Executor::Impl (src/executor.cpp:39-78): the plugin, its
// plans (shared_ptr<const AxisPlan> built by the reference planner) and its
// calls stay as they are.
//
// Plans given to prepare() are imported once (dsmvc_gb_plan_import: copied,
// validated like AxisPlan::check_valid) and kept for the executor's life,
// keyed by plan identity together with the caller's shared_ptr, like the
// reference's prepared set (src/cuda/cuda_executor.cpp:2490-2525).  A plan
// that was not prepared is imported for the one call.  Errors arrive as the
// reference's exception types: std::invalid_argument, std::length_error,
// std::runtime_error.  The first executor installs the CUDA domain's
// registrar in the engine's host block registry (include/dsmvc/
// host_blocks.hpp), as the reference's CUDA runtime does, so that the
// plugin's frame-pool blocks are page-locked for direct transfers.  GPU
// frames exported by a Vulkan core need graphics interop, which this
// backend does not have: those calls throw.
#pragma once

#include <dsmvc/engine.hpp>

#include <cstddef>
#include <cstdint>
#include <memory>

namespace dsmvc::gb300_detail {

[[nodiscard]] bool backend_available() noexcept;

class Gb300Executor {
public:
    Gb300Executor();
    // For GPU frames of a core: unsupported here (no graphics interop).
    explicit Gb300Executor(const std::uint8_t device_uuid[16]);
    ~Gb300Executor();
    Gb300Executor(const Gb300Executor &) noexcept = default;
    Gb300Executor &operator=(const Gb300Executor &) noexcept = default;
    Gb300Executor(Gb300Executor &&) noexcept = default;
    Gb300Executor &operator=(Gb300Executor &&) noexcept = default;

    [[nodiscard]] const char *name() const noexcept;
    [[nodiscard]] bool input_cache_enabled() const noexcept;
    void prepare(std::shared_ptr<const AxisPlan> plan) const;
    void seal() const;

    void inverse_rows(const AxisPlan &plan,
                      const float *input, std::ptrdiff_t input_row_stride,
                      float *output, std::ptrdiff_t output_row_stride,
                      std::int32_t row_count,
                      std::shared_ptr<const void> input_lifetime) const;
    void inverse_columns(const AxisPlan &plan,
                         const float *input, std::ptrdiff_t input_row_stride,
                         float *output, std::ptrdiff_t output_row_stride,
                         std::int32_t column_count,
                         std::shared_ptr<const void> input_lifetime) const;
    void inverse_2d(const AxisPlan &horizontal, const AxisPlan &vertical,
                    const float *input, std::ptrdiff_t input_row_stride,
                    float *output, std::ptrdiff_t output_row_stride,
                    std::shared_ptr<const void> input_lifetime) const;
    void inverse_2d_u8(const AxisPlan &horizontal, const AxisPlan &vertical,
                       const std::uint8_t *input, std::ptrdiff_t input_row_stride,
                       std::uint8_t *output, std::ptrdiff_t output_row_stride,
                       const IntegerConversion &conversion,
                       std::shared_ptr<const void> input_lifetime) const;
    void inverse_2d_u16(const AxisPlan &horizontal, const AxisPlan &vertical,
                        const std::uint16_t *input, std::ptrdiff_t input_row_stride,
                        std::uint16_t *output, std::ptrdiff_t output_row_stride,
                        const IntegerConversion &conversion,
                        std::shared_ptr<const void> input_lifetime) const;

    // GPU frames exported by a Vulkan core (ExportedPlane): not supported.
    [[nodiscard]] bool has_exported_semaphore(std::uint64_t semaphore) const;
    [[nodiscard]] bool import_exported_semaphore(std::uint64_t semaphore, int handle_type,
                                                 std::intptr_t handle) const;
    void inverse_rows_exported(const AxisPlan &plan, const ExportedPlane &input,
                               const ExportedPlane &output, std::int32_t row_count) const;
    void inverse_columns_exported(const AxisPlan &plan, const ExportedPlane &input,
                                  const ExportedPlane &output, std::int32_t column_count) const;
    void inverse_2d_exported(const AxisPlan &horizontal, const AxisPlan &vertical,
                             const ExportedPlane &input, const ExportedPlane &output) const;
    void inverse_2d_u8_exported(const AxisPlan &horizontal, const AxisPlan &vertical,
                                const ExportedPlane &input, const ExportedPlane &output,
                                const IntegerConversion &conversion) const;
    void inverse_2d_u16_exported(const AxisPlan &horizontal, const AxisPlan &vertical,
                                 const ExportedPlane &input, const ExportedPlane &output,
                                 const IntegerConversion &conversion) const;

    // Imports `plan` into a plan handle of the GB300 C ABI (owned by the
    // caller, released with dsmvc_gb_plan_release).  Exposed for tests and
    // for callers that mix this class with direct C-ABI calls.
    [[nodiscard]] static void *import_plan(const AxisPlan &plan);

private:
    struct Impl;
    std::shared_ptr<Impl> impl_;
};

} // namespace dsmvc::gb300_detail
