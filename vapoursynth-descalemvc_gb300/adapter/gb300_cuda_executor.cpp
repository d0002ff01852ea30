// Drop-in CUDA backend for the reference engine over the GB300 executor's
// C ABI (see gb300_cuda_executor.hpp).  Built against the reference's
// include/dsmvc/engine.hpp and linked with libdsmvc_gb300.so.
#include "gb300_cuda_executor.hpp"

#include "dsmvc_gb300.h"

#include <dsmvc/host_blocks.hpp>

#include <cstdlib>
#include <mutex>
#include <stdexcept>
#include <string>
#include <string_view>
#include <unordered_map>

namespace dsmvc::gb300_detail {
namespace {

// The reference's exception types for the C ABI's status codes.
void check(int status) {
    if (status == DSMVC_GB_OK) return;
    const std::string message = std::string("dsmvc: ") + dsmvc_gb_last_error();
    switch (status) {
    case DSMVC_GB_INVALID_ARGUMENT: throw std::invalid_argument(message);
    case DSMVC_GB_LENGTH_ERROR: throw std::length_error(message);
    default: throw std::runtime_error(message);
    }
}

struct PlanHandle {
    dsmvc_gb_plan *handle = nullptr;
    explicit PlanHandle(dsmvc_gb_plan *h) : handle(h) {}
    PlanHandle(const PlanHandle &) = delete;
    PlanHandle &operator=(const PlanHandle &) = delete;
    ~PlanHandle() { dsmvc_gb_plan_release(handle); }
};

dsmvc_gb_plan *import(const AxisPlan &p) {
    dsmvc_gb_plan_arrays a{};
    a.source_size = p.source_size;
    a.destination_size = p.destination_size;
    a.support = p.support;
    a.half_bandwidth = p.half_bandwidth;
    a.active_length = p.active_length;
    a.shift = p.shift;
    a.normal_rcond = p.normal_rcond;
    a.normal_inf_norm = p.normal_inf_norm;
    a.transpose_offsets = p.transpose_offsets.data();
    a.transpose_offsets_count = p.transpose_offsets.size();
    a.transpose_indices = p.transpose_indices.data();
    a.transpose_indices_count = p.transpose_indices.size();
    a.transpose_weights = p.transpose_weights.data();
    a.transpose_weights_count = p.transpose_weights.size();
    a.lower_ld = p.lower_ld.data();
    a.lower_ld_count = p.lower_ld.size();
    a.upper_l = p.upper_l.data();
    a.upper_l_count = p.upper_l.size();
    a.inverse_diagonal = p.inverse_diagonal.data();
    a.inverse_diagonal_count = p.inverse_diagonal.size();
    a.transpose_weights_f64 = p.transpose_weights_f64.data();
    a.transpose_weights_f64_count = p.transpose_weights_f64.size();
    a.normal_bands_f64 = p.normal_bands_f64.data();
    a.normal_bands_f64_count = p.normal_bands_f64.size();
    a.ldlt_bands_f64 = p.ldlt_bands_f64.data();
    a.ldlt_bands_f64_count = p.ldlt_bands_f64.size();
    a.inverse_diagonal_f64 = p.inverse_diagonal_f64.data();
    a.inverse_diagonal_f64_count = p.inverse_diagonal_f64.size();
    dsmvc_gb_plan *out = nullptr;
    check(dsmvc_gb_plan_import(&a, &out));
    return out;
}

[[noreturn]] void no_exported_frames() {
    throw std::runtime_error(
        "dsmvc: GPU frames exported by a Vulkan core need graphics interop, which the GB300 "
        "backend does not provide; use host frames");
}

// Direct transfers from and to the plugin's frame-pool blocks.  The
// reference plugin reports its blocks to the engine's host block registry
// (include/dsmvc/host_blocks.hpp, src/vs_frame_memory.cpp), and only while
// a registrar is installed for the CUDA domain (vs_frame_memory.cpp:155);
// the reference's CUDA backend installs one with its runtime
// (src/cuda/cuda_executor.cpp:198-202, 1327-1361, 1425-1441).  This one
// page-locks a block through dsmvc_gb_host_register, after which the GB300
// executor's copies from and to planes inside it run as DMA.  It is
// installed with the first executor and stays for the process's life, like
// the reference's shared runtime; DSMVC_CUDA_DIRECT_IO=0 or an explicit
// DSMVC_CUDA_HOST_TRANSFER leave it out, as in the reference.
bool block_direct_io_requested() noexcept {
    const char *direct = std::getenv("DSMVC_CUDA_DIRECT_IO");
    return !(direct && std::string_view{direct} == "0") && !std::getenv("DSMVC_CUDA_HOST_TRANSFER");
}

host_blocks::Registered register_block(void *base, std::size_t size) noexcept {
    std::int32_t outcome = -1;
    if (dsmvc_gb_host_register(base, static_cast<std::int64_t>(size), &outcome) != DSMVC_GB_OK) return {};
    if (outcome == 0) return {host_blocks::Outcome::owned, {}};
    if (outcome == 1) return {host_blocks::Outcome::foreign, {}};
    return {};
}

void unregister_block(void *base, std::size_t, const std::shared_ptr<void> &) noexcept {
    (void)dsmvc_gb_host_unregister(base);
}

struct DirectBlocks {
    bool installed = false;
    DirectBlocks() {
        if (!block_direct_io_requested()) return;
        host_blocks::install(host_blocks::Domain::cuda, {&register_block, &unregister_block});
        installed = true;
    }
    ~DirectBlocks() {
        if (installed) host_blocks::uninstall(host_blocks::Domain::cuda);
    }
    DirectBlocks(const DirectBlocks &) = delete;
    DirectBlocks &operator=(const DirectBlocks &) = delete;
};

} // namespace

bool backend_available() noexcept { return dsmvc_gb_cuda_available() != 0; }

struct Gb300Executor::Impl {
    dsmvc_gb_executor *executor = nullptr;
    std::mutex mutex;
    struct Prepared {
        std::shared_ptr<const AxisPlan> owner;
        std::shared_ptr<PlanHandle> handle;
    };
    std::unordered_map<const AxisPlan *, Prepared> prepared;

    Impl() {
        check(dsmvc_gb_executor_create(-1, &executor));
        static DirectBlocks direct_blocks;
    }
    ~Impl() { dsmvc_gb_executor_destroy(executor); }

    // The handle of a prepared plan, or a one-call import.
    std::shared_ptr<PlanHandle> handle_of(const AxisPlan &plan) {
        {
            std::scoped_lock lock(mutex);
            const auto found = prepared.find(&plan);
            if (found != prepared.end()) return found->second.handle;
        }
        return std::make_shared<PlanHandle>(import(plan));
    }
};

Gb300Executor::Gb300Executor() : impl_(std::make_shared<Impl>()) {}

Gb300Executor::Gb300Executor(const std::uint8_t *) { no_exported_frames(); }

Gb300Executor::~Gb300Executor() = default;

const char *Gb300Executor::name() const noexcept { return "cuda"; }

bool Gb300Executor::input_cache_enabled() const noexcept { return false; }

void Gb300Executor::prepare(std::shared_ptr<const AxisPlan> plan) const {
    if (!plan) throw std::invalid_argument("dsmvc: cannot prepare a null plan");
    {
        std::scoped_lock lock(impl_->mutex);
        if (impl_->prepared.count(plan.get())) return;
    }
    auto handle = std::make_shared<PlanHandle>(import(*plan));
    check(dsmvc_gb_prepare(impl_->executor, handle->handle));
    std::scoped_lock lock(impl_->mutex);
    impl_->prepared.emplace(plan.get(), Impl::Prepared{std::move(plan), std::move(handle)});
}

void Gb300Executor::seal() const { check(dsmvc_gb_seal(impl_->executor)); }

void Gb300Executor::inverse_rows(const AxisPlan &plan, const float *input, std::ptrdiff_t input_row_stride,
                                 float *output, std::ptrdiff_t output_row_stride, std::int32_t row_count,
                                 std::shared_ptr<const void>) const {
    const auto h = impl_->handle_of(plan);
    check(dsmvc_gb_inverse_rows(impl_->executor, h->handle, input, input_row_stride, output,
                                output_row_stride, row_count));
}

void Gb300Executor::inverse_columns(const AxisPlan &plan, const float *input, std::ptrdiff_t input_row_stride,
                                    float *output, std::ptrdiff_t output_row_stride,
                                    std::int32_t column_count, std::shared_ptr<const void>) const {
    const auto h = impl_->handle_of(plan);
    check(dsmvc_gb_inverse_columns(impl_->executor, h->handle, input, input_row_stride, output,
                                   output_row_stride, column_count));
}

void Gb300Executor::inverse_2d(const AxisPlan &horizontal, const AxisPlan &vertical, const float *input,
                               std::ptrdiff_t input_row_stride, float *output, std::ptrdiff_t output_row_stride,
                               std::shared_ptr<const void>) const {
    const auto h = impl_->handle_of(horizontal);
    const auto v = impl_->handle_of(vertical);
    check(dsmvc_gb_inverse_2d(impl_->executor, h->handle, v->handle, input, input_row_stride, output,
                              output_row_stride));
}

void Gb300Executor::inverse_2d_u8(const AxisPlan &horizontal, const AxisPlan &vertical,
                                  const std::uint8_t *input, std::ptrdiff_t input_row_stride,
                                  std::uint8_t *output, std::ptrdiff_t output_row_stride,
                                  const IntegerConversion &c, std::shared_ptr<const void>) const {
    const auto h = impl_->handle_of(horizontal);
    const auto v = impl_->handle_of(vertical);
    const dsmvc_gb_conversion conv{c.input_offset, c.input_scale, c.output_scale, c.output_offset,
                                   c.output_maximum};
    check(dsmvc_gb_inverse_2d_u8(impl_->executor, h->handle, v->handle, input, input_row_stride, output,
                                 output_row_stride, &conv));
}

void Gb300Executor::inverse_2d_u16(const AxisPlan &horizontal, const AxisPlan &vertical,
                                   const std::uint16_t *input, std::ptrdiff_t input_row_stride,
                                   std::uint16_t *output, std::ptrdiff_t output_row_stride,
                                   const IntegerConversion &c, std::shared_ptr<const void>) const {
    const auto h = impl_->handle_of(horizontal);
    const auto v = impl_->handle_of(vertical);
    const dsmvc_gb_conversion conv{c.input_offset, c.input_scale, c.output_scale, c.output_offset,
                                   c.output_maximum};
    check(dsmvc_gb_inverse_2d_u16(impl_->executor, h->handle, v->handle, input, input_row_stride, output,
                                  output_row_stride, &conv));
}

bool Gb300Executor::has_exported_semaphore(std::uint64_t) const { return false; }

bool Gb300Executor::import_exported_semaphore(std::uint64_t, int, std::intptr_t handle) const {
    // The handle is consumed whatever the outcome (engine.hpp:367-370).
    ExportedPlane plane;
    plane.handle = handle;
    close_exported_plane(plane);
    return false;
}

void Gb300Executor::inverse_rows_exported(const AxisPlan &, const ExportedPlane &, const ExportedPlane &,
                                          std::int32_t) const {
    no_exported_frames();
}

void Gb300Executor::inverse_columns_exported(const AxisPlan &, const ExportedPlane &, const ExportedPlane &,
                                             std::int32_t) const {
    no_exported_frames();
}

void Gb300Executor::inverse_2d_exported(const AxisPlan &, const AxisPlan &, const ExportedPlane &,
                                        const ExportedPlane &) const {
    no_exported_frames();
}

void Gb300Executor::inverse_2d_u8_exported(const AxisPlan &, const AxisPlan &, const ExportedPlane &,
                                           const ExportedPlane &, const IntegerConversion &) const {
    no_exported_frames();
}

void Gb300Executor::inverse_2d_u16_exported(const AxisPlan &, const AxisPlan &, const ExportedPlane &,
                                            const ExportedPlane &, const IntegerConversion &) const {
    no_exported_frames();
}

void *Gb300Executor::import_plan(const AxisPlan &plan) { return import(plan); }

} // namespace dsmvc::gb300_detail
