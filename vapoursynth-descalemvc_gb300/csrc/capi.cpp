// extern "C" boundary (include/dsmvc_gb300.h): converts C++ exceptions to
// status codes plus a thread-local message; no exception crosses the ABI.
#include "../../include/dsmvc_gb300.h"

#include "executor.hpp"
#include "host_blocks.hpp"
#include "noalloc.hpp"
#include "peak.hpp"
#include "server.hpp"
#include "sweep.hpp"
#include "planner.hpp"
#include "stream.cuh"
#include "stream_plan.hpp"

#include <algorithm>
#include <atomic>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include <cstdio>
#include <new>
#include <stdexcept>
#include <string>

struct dsmvc_gb_plan {
    std::shared_ptr<const dsmvc_gb::AxisPlan> plan;
    dsmvc_gb::AxisRequest request;
    // Imported plans (dsmvc_gb_plan_import) carry no request.
    bool has_request = true;
};

struct dsmvc_gb_executor {
    dsmvc_gb::Executor executor;
    explicit dsmvc_gb_executor(int device) : executor(device) {}
};

namespace {

thread_local std::string g_error;

template <class F>
int guarded(F &&f) noexcept {
    try {
        g_error.clear();
        f();
        return DSMVC_GB_OK;
    } catch (const std::invalid_argument &e) {
        g_error = e.what();
        return DSMVC_GB_INVALID_ARGUMENT;
    } catch (const std::length_error &e) {
        g_error = e.what();
        return DSMVC_GB_LENGTH_ERROR;
    } catch (const std::out_of_range &e) {
        g_error = e.what();
        return DSMVC_GB_LENGTH_ERROR;
    } catch (const std::bad_alloc &) {
        g_error = "out of host memory";
        return DSMVC_GB_OUT_OF_MEMORY;
    } catch (const std::logic_error &e) {
        g_error = e.what();
        return DSMVC_GB_INVALID_ARGUMENT;
    } catch (const std::runtime_error &e) {
        g_error = e.what();
        const std::string m = e.what();
        if (m.rfind("CUDA", 0) == 0) {
            return m.find("out of memory") != std::string::npos ? DSMVC_GB_OUT_OF_MEMORY
                                                                : DSMVC_GB_CUDA_ERROR;
        }
        if (m.find("requires an available CUDA device") != std::string::npos) return DSMVC_GB_UNAVAILABLE;
        return DSMVC_GB_RUNTIME_ERROR;
    } catch (...) {
        g_error = "unknown error";
        return DSMVC_GB_RUNTIME_ERROR;
    }
}

dsmvc_gb::AxisRequest to_request(const dsmvc_gb_axis_request *r) {
    if (!r) throw std::invalid_argument("request is null");
    if (r->kernel < 0 || r->kernel > DSMVC_GB_CUSTOM) throw std::invalid_argument("kernel kind is invalid");
    if (r->border < 0 || r->border > DSMVC_GB_MIRROR) throw std::invalid_argument("padding mode is invalid");
    if (r->f64_mode < 0 || r->f64_mode > DSMVC_GB_F64_FORCE) throw std::invalid_argument("f64 mode is invalid");
    dsmvc_gb::AxisRequest q;
    q.source_size = r->source_size;
    q.destination_size = r->destination_size;
    q.active_length = r->active_length;
    q.shift = r->shift;
    q.kernel.kind = static_cast<dsmvc_gb::KernelKind>(r->kernel);
    q.kernel.taps = r->taps;
    q.kernel.b = r->b;
    q.kernel.c = r->c;
    q.kernel.blur = r->blur;
    q.border = static_cast<dsmvc_gb::BorderMode>(r->border);
    q.f64_mode = static_cast<dsmvc_gb::F64Mode>(r->f64_mode);
    return q;
}

dsmvc_gb::CustomKernel to_custom(dsmvc_gb_custom_kernel fn, void *user) {
    if (!fn) return {};
    return [fn, user](double x) { return fn(x, user); };
}

const dsmvc_gb::AxisPlan &plan_of(const dsmvc_gb_plan *p) {
    if (!p || !p->plan) throw std::invalid_argument("plan is null");
    return *p->plan;
}

dsmvc_gb::Executor &exec_of(dsmvc_gb_executor *e) {
    if (!e) throw std::invalid_argument("executor is null");
    return e->executor;
}

dsmvc_gb::IntegerConversion to_conversion(const dsmvc_gb_conversion *c) {
    if (!c) throw std::invalid_argument("conversion is null");
    return {c->input_offset, c->input_scale, c->output_scale, c->output_offset, c->output_maximum};
}

} // namespace

extern "C" {

const char *dsmvc_gb_last_error(void) { return g_error.c_str(); }

int dsmvc_gb_abi_version(void) { return DSMVC_GB_ABI_VERSION; }

int dsmvc_gb_cuda_available(void) {
    int count = 0;
    return cudaGetDeviceCount(&count) == cudaSuccess && count > 0 ? 1 : 0;
}

int dsmvc_gb_plan_build(const dsmvc_gb_axis_request *request, dsmvc_gb_custom_kernel custom,
                        void *user, dsmvc_gb_plan **out) {
    return guarded([&] {
        if (!out) throw std::invalid_argument("output handle is null");
        *out = nullptr;
        auto q = to_request(request);
        auto plan = std::make_shared<const dsmvc_gb::AxisPlan>(
            dsmvc_gb::build_axis_plan(q, to_custom(custom, user)));
        *out = new dsmvc_gb_plan{std::move(plan), q};
    });
}

int dsmvc_gb_plan_get_or_build(const dsmvc_gb_axis_request *request, dsmvc_gb_custom_kernel custom,
                               void *user, dsmvc_gb_plan **out) {
    return guarded([&] {
        if (!out) throw std::invalid_argument("output handle is null");
        *out = nullptr;
        auto q = to_request(request);
        auto plan = dsmvc_gb::get_or_build_axis_plan(q, to_custom(custom, user));
        *out = new dsmvc_gb_plan{std::move(plan), q};
    });
}

void dsmvc_gb_plan_release(dsmvc_gb_plan *plan) { delete plan; }

int dsmvc_gb_plan_build_many(const dsmvc_gb_axis_request *requests, int32_t count, int32_t threads,
                             dsmvc_gb_plan **out) {
    return guarded([&] {
        if (count < 0 || (count > 0 && (!requests || !out))) throw std::invalid_argument("invalid plan list");
        std::vector<dsmvc_gb::AxisRequest> qs;
        qs.reserve(static_cast<std::size_t>(count));
        for (int32_t i = 0; i < count; ++i) qs.push_back(to_request(&requests[i]));
        for (int32_t i = 0; i < count; ++i) out[i] = nullptr;
        std::vector<std::shared_ptr<const dsmvc_gb::AxisPlan>> built(static_cast<std::size_t>(count));
        std::vector<std::string> errors(static_cast<std::size_t>(count));
        std::atomic<int32_t> next{0};
        auto worker = [&] {
            for (int32_t i = next++; i < count; i = next++) {
                try {
                    built[static_cast<std::size_t>(i)] = std::make_shared<const dsmvc_gb::AxisPlan>(
                        dsmvc_gb::build_axis_plan(qs[static_cast<std::size_t>(i)]));
                } catch (const std::exception &e) {
                    errors[static_cast<std::size_t>(i)] = e.what();
                }
            }
        };
        unsigned n = threads > 0 ? static_cast<unsigned>(threads) : std::thread::hardware_concurrency();
        n = std::max(1U, std::min<unsigned>(n, static_cast<unsigned>(std::max(count, 1))));
        std::vector<std::thread> pool;
        for (unsigned t = 1; t < n; ++t) pool.emplace_back(worker);
        worker();
        for (auto &t : pool) t.join();
        for (int32_t i = 0; i < count; ++i)
            if (!errors[static_cast<std::size_t>(i)].empty())
                throw std::invalid_argument("plan " + std::to_string(i) + ": " + errors[static_cast<std::size_t>(i)]);
        for (int32_t i = 0; i < count; ++i)
            out[i] = new dsmvc_gb_plan{std::move(built[static_cast<std::size_t>(i)]), qs[static_cast<std::size_t>(i)]};
    });
}

int dsmvc_gb_plan_build_many_device(const dsmvc_gb_axis_request *requests, int32_t count, int32_t device,
                                    int32_t threads, dsmvc_gb_plan **out) {
    return guarded([&] {
        if (count < 0 || (count > 0 && (!requests || !out))) throw std::invalid_argument("invalid plan list");
        std::vector<dsmvc_gb::AxisRequest> qs;
        qs.reserve(static_cast<std::size_t>(count));
        for (int32_t i = 0; i < count; ++i) qs.push_back(to_request(&requests[i]));
        for (int32_t i = 0; i < count; ++i) out[i] = nullptr;
        auto plans = dsmvc_gb::build_axis_plans_on_device(qs, device, threads);
        for (int32_t i = 0; i < count; ++i)
            out[i] = new dsmvc_gb_plan{std::make_shared<const dsmvc_gb::AxisPlan>(
                                           std::move(plans[static_cast<std::size_t>(i)])),
                                       qs[static_cast<std::size_t>(i)]};
    });
}

int dsmvc_gb_plan_get_info(const dsmvc_gb_plan *plan, dsmvc_gb_plan_info *out) {
    return guarded([&] {
        const auto &p = plan_of(plan);
        if (!out) throw std::invalid_argument("output is null");
        out->source_size = p.source_size;
        out->destination_size = p.destination_size;
        out->support = p.support;
        out->half_bandwidth = p.half_bandwidth;
        out->requires_float64 = p.requires_float64() ? 1 : 0;
        out->max_row_entries = p.max_row_entries;
        out->active_length = p.active_length;
        out->shift = p.shift;
        out->normal_rcond = p.normal_rcond;
        out->normal_inf_norm = p.normal_inf_norm;
        out->nonzeros = p.transpose_indices.size();
        out->storage_bytes = p.storage_bytes();
    });
}

int dsmvc_gb_plan_get_array(const dsmvc_gb_plan *plan, int32_t which, const void **data,
                            uint64_t *count) {
    return guarded([&] {
        const auto &p = plan_of(plan);
        if (!data || !count) throw std::invalid_argument("output is null");
        switch (which) {
        case 0: *data = p.transpose_offsets.data(); *count = p.transpose_offsets.size(); break;
        case 1: *data = p.transpose_indices.data(); *count = p.transpose_indices.size(); break;
        case 2: *data = p.transpose_weights.data(); *count = p.transpose_weights.size(); break;
        case 3: *data = p.lower_ld.data(); *count = p.lower_ld.size(); break;
        case 4: *data = p.upper_l.data(); *count = p.upper_l.size(); break;
        case 5: *data = p.inverse_diagonal.data(); *count = p.inverse_diagonal.size(); break;
        case 6: *data = p.transpose_weights_f64.data(); *count = p.transpose_weights_f64.size(); break;
        case 7: *data = p.normal_bands_f64.data(); *count = p.normal_bands_f64.size(); break;
        case 8: *data = p.ldlt_bands_f64.data(); *count = p.ldlt_bands_f64.size(); break;
        case 9: *data = p.inverse_diagonal_f64.data(); *count = p.inverse_diagonal_f64.size(); break;
        default: throw std::invalid_argument("plan array index is invalid");
        }
    });
}

int dsmvc_gb_plan_import(const dsmvc_gb_plan_arrays *a, dsmvc_gb_plan **out) {
    return guarded([&] {
        if (!out) throw std::invalid_argument("output handle is null");
        *out = nullptr;
        if (!a) throw std::invalid_argument("plan arrays are null");
        auto copy = [](const auto *data, std::uint64_t count, auto &dst, const char *name) {
            if (count > 0 && !data) throw std::invalid_argument(std::string("plan array ") + name + " is null");
            if (count > (std::uint64_t{1} << 40)) throw std::length_error(std::string("plan array ") + name + " is too large");
            dst.assign(data, data + count);
        };
        dsmvc_gb::AxisPlan p;
        p.source_size = a->source_size;
        p.destination_size = a->destination_size;
        p.support = a->support;
        p.half_bandwidth = a->half_bandwidth;
        p.active_length = a->active_length;
        p.shift = a->shift;
        p.normal_rcond = a->normal_rcond;
        p.normal_inf_norm = a->normal_inf_norm;
        copy(a->transpose_offsets, a->transpose_offsets_count, p.transpose_offsets, "transpose_offsets");
        copy(a->transpose_indices, a->transpose_indices_count, p.transpose_indices, "transpose_indices");
        copy(a->transpose_weights, a->transpose_weights_count, p.transpose_weights, "transpose_weights");
        copy(a->lower_ld, a->lower_ld_count, p.lower_ld, "lower_ld");
        copy(a->upper_l, a->upper_l_count, p.upper_l, "upper_l");
        copy(a->inverse_diagonal, a->inverse_diagonal_count, p.inverse_diagonal, "inverse_diagonal");
        copy(a->transpose_weights_f64, a->transpose_weights_f64_count, p.transpose_weights_f64,
             "transpose_weights_f64");
        copy(a->normal_bands_f64, a->normal_bands_f64_count, p.normal_bands_f64, "normal_bands_f64");
        copy(a->ldlt_bands_f64, a->ldlt_bands_f64_count, p.ldlt_bands_f64, "ldlt_bands_f64");
        copy(a->inverse_diagonal_f64, a->inverse_diagonal_f64_count, p.inverse_diagonal_f64,
             "inverse_diagonal_f64");
        if (p.transpose_offsets.empty() || !p.valid())
            throw std::invalid_argument("imported axis plan is invalid");
        std::int32_t widest = 0;
        for (std::size_t j = 0; j + 1 < p.transpose_offsets.size(); ++j)
            widest = std::max<std::int32_t>(widest, static_cast<std::int32_t>(p.transpose_offsets[j + 1]
                                                                              - p.transpose_offsets[j]));
        p.max_row_entries = widest;
        p.validated = true;
        dsmvc_gb::AxisRequest q;
        q.source_size = p.source_size;
        q.destination_size = p.destination_size;
        q.active_length = p.active_length;
        q.shift = p.shift;
        q.kernel.kind = dsmvc_gb::KernelKind::custom;
        q.f64_mode = p.requires_float64() ? dsmvc_gb::F64Mode::float64_only : dsmvc_gb::F64Mode::automatic;
        *out = new dsmvc_gb_plan{std::make_shared<const dsmvc_gb::AxisPlan>(std::move(p)), q, false};
    });
}

int dsmvc_gb_plan_hashes(const dsmvc_gb_plan *plan, const dsmvc_gb_axis_request *request,
                         uint64_t *f32_hash, uint64_t *complete_hash) {
    return guarded([&] {
        const auto &p = plan_of(plan);
        if (!request && !plan->has_request)
            throw std::invalid_argument("an imported plan carries no request: pass one for its hashes");
        const auto q = request ? to_request(request) : plan->request;
        if (f32_hash) *f32_hash = dsmvc_gb::f32_plan_hash(q, p);
        if (complete_hash) *complete_hash = dsmvc_gb::complete_plan_hash(q, p);
    });
}

int dsmvc_gb_plan_stream_info(const dsmvc_gb_plan *plan, dsmvc_gb_stream_info *info, float *forward,
                              uint64_t forward_capacity, float *backward, uint64_t backward_capacity) {
    return guarded([&] {
        const auto &p = plan_of(plan);
        if (!info) throw std::invalid_argument("output is null");
        const auto pack = dsmvc_gb::pack_stream_plan(p, dsmvc_gb::kStreamChunk, dsmvc_gb::kStreamRing,
                                                     dsmvc_gb::stream_supports(p.half_bandwidth),
                                                     dsmvc_gb::tsolve_supports(p.half_bandwidth));
        *info = {};
        info->eligible = pack.eligible ? 1 : 0;
        info->window = pack.window;
        info->forward_stride = pack.forward_stride;
        info->backward_stride = pack.backward_stride;
        info->ring_ok_u16 = pack.ring_ok_u16 ? 1 : 0;
        info->ring_ok_u8 = pack.ring_ok_u8 ? 1 : 0;
        info->ring_ok_transposed = pack.ring_ok_transposed ? 1 : 0;
        info->exact = pack.exact ? 1 : 0;
        info->segmentable = pack.segmentable ? 1 : 0;
        info->forward_transfer = pack.forward_transfer;
        info->group_union = pack.group_union;
        info->group_stride = pack.group_stride;
        const auto pack64 = dsmvc_gb::pack_stream_plan64(p, dsmvc_gb::kStreamChunk, dsmvc_gb::kStreamRing,
                                                         dsmvc_gb::tsolve_supports(p.half_bandwidth));
        info->f64_eligible = pack64.eligible ? 1 : 0;
        info->f64_segmentable = pack64.segmentable ? 1 : 0;
        info->f64_margin = pack64.margin;
        info->exact_margin = pack.exact_margin;
        info->exact_margin_transfer = pack.exact_margin_transfer;
        info->f64_margin_transfer = pack64.margin_transfer;
        info->chunk = dsmvc_gb::kStreamChunk;
        info->ring = dsmvc_gb::kStreamRing;
        info->backward_transfer = pack.backward_transfer;
        std::snprintf(info->reason, sizeof(info->reason), "%s", pack.reason.c_str());
        if (forward && forward_capacity >= pack.forward.size())
            std::copy(pack.forward.begin(), pack.forward.end(), forward);
        if (backward && backward_capacity >= pack.backward.size())
            std::copy(pack.backward.begin(), pack.backward.end(), backward);
    });
}

int dsmvc_gb_plan_stream_groups(const dsmvc_gb_plan *plan, float *out, uint64_t capacity, uint64_t *count) {
    return guarded([&] {
        const auto &p = plan_of(plan);
        const auto pack = dsmvc_gb::pack_stream_plan(p, dsmvc_gb::kStreamChunk, dsmvc_gb::kStreamRing,
                                                     dsmvc_gb::stream_supports(p.half_bandwidth),
                                                     dsmvc_gb::tsolve_supports(p.half_bandwidth));
        if (count) *count = pack.forward_groups.size();
        if (out) {
            if (capacity < pack.forward_groups.size()) throw std::length_error("group buffer too small");
            std::copy(pack.forward_groups.begin(), pack.forward_groups.end(), out);
        }
    });
}

int dsmvc_gb_planner_cache_stats(dsmvc_gb_planner_stats *out) {
    return guarded([&] {
        if (!out) throw std::invalid_argument("output is null");
        const auto s = dsmvc_gb::planner_cache_stats();
        out->plan_hits = s.plan_hits;
        out->plan_builds = s.plan_builds;
        out->plan_entries = s.plan_entries;
        out->plan_resident_bytes = s.plan_resident_bytes;
    });
}

void dsmvc_gb_clear_planner_caches(void) { dsmvc_gb::clear_planner_caches(); }

int dsmvc_gb_executor_create(int32_t device, dsmvc_gb_executor **out) {
    return guarded([&] {
        if (!out) throw std::invalid_argument("output handle is null");
        *out = nullptr;
        *out = new dsmvc_gb_executor(device);
    });
}

void dsmvc_gb_executor_destroy(dsmvc_gb_executor *executor) { delete executor; }

int dsmvc_gb_prepare(dsmvc_gb_executor *executor, const dsmvc_gb_plan *plan) {
    return guarded([&] {
        plan_of(plan);
        exec_of(executor).prepare(plan->plan);
    });
}

int dsmvc_gb_prepare_many(dsmvc_gb_executor *executor, const dsmvc_gb_plan *const *plans, int32_t count) {
    return guarded([&] {
        if (count < 0 || (count > 0 && !plans)) throw std::invalid_argument("invalid plan list");
        std::vector<std::shared_ptr<const dsmvc_gb::AxisPlan>> list;
        list.reserve(static_cast<std::size_t>(count));
        for (int32_t i = 0; i < count; ++i) {
            plan_of(plans[i]);
            list.push_back(plans[i]->plan);
        }
        exec_of(executor).prepare_many(list);
    });
}

int dsmvc_gb_seal(dsmvc_gb_executor *executor) {
    return guarded([&] { exec_of(executor).seal(); });
}

int dsmvc_gb_executor_get_stats(dsmvc_gb_executor *executor, dsmvc_gb_executor_stats *out) {
    return guarded([&] {
        if (!out) throw std::invalid_argument("output is null");
        const auto s = exec_of(executor).stats();
        out->launches = s.launches;
        out->plane_tasks = s.plane_tasks;
        out->plan_uploads = s.plan_uploads;
        out->device_plan_bytes = s.device_plan_bytes;
        out->workspace_bytes = s.workspace_bytes;
        out->plan_cache_hits = s.plan_cache_hits;
        out->plan_cache_misses = s.plan_cache_misses;
        out->plan_cache_evictions = s.plan_cache_evictions;
        out->plan_cache_bytes = s.plan_cache_bytes;
        out->compile_reuses = s.compile_reuses;
    });
}

int dsmvc_gb_inverse_rows(dsmvc_gb_executor *executor, const dsmvc_gb_plan *plan,
                          const float *input, int64_t input_stride, float *output,
                          int64_t output_stride, int32_t rows) {
    return guarded([&] {
        exec_of(executor).inverse_rows(plan_of(plan), input, input_stride, output, output_stride, rows,
                                       plan->plan);
    });
}

int dsmvc_gb_inverse_columns(dsmvc_gb_executor *executor, const dsmvc_gb_plan *plan,
                             const float *input, int64_t input_stride, float *output,
                             int64_t output_stride, int32_t columns) {
    return guarded([&] {
        exec_of(executor).inverse_columns(plan_of(plan), input, input_stride, output, output_stride,
                                          columns, plan->plan);
    });
}

int dsmvc_gb_inverse_2d(dsmvc_gb_executor *executor, const dsmvc_gb_plan *horizontal,
                        const dsmvc_gb_plan *vertical, const float *input, int64_t input_stride,
                        float *output, int64_t output_stride) {
    return guarded([&] {
        exec_of(executor).inverse_2d(plan_of(horizontal), plan_of(vertical), dsmvc_gb::dev::Sample::f32,
                                     input, input_stride, output, output_stride, {}, horizontal->plan,
                                     vertical->plan);
    });
}

int dsmvc_gb_inverse_2d_u8(dsmvc_gb_executor *executor, const dsmvc_gb_plan *horizontal,
                           const dsmvc_gb_plan *vertical, const uint8_t *input, int64_t input_stride,
                           uint8_t *output, int64_t output_stride,
                           const dsmvc_gb_conversion *conversion) {
    return guarded([&] {
        exec_of(executor).inverse_2d(plan_of(horizontal), plan_of(vertical), dsmvc_gb::dev::Sample::u8,
                                     input, input_stride, output, output_stride,
                                     to_conversion(conversion), horizontal->plan, vertical->plan);
    });
}

int dsmvc_gb_inverse_2d_u16(dsmvc_gb_executor *executor, const dsmvc_gb_plan *horizontal,
                            const dsmvc_gb_plan *vertical, const uint16_t *input,
                            int64_t input_stride, uint16_t *output, int64_t output_stride,
                            const dsmvc_gb_conversion *conversion) {
    return guarded([&] {
        exec_of(executor).inverse_2d(plan_of(horizontal), plan_of(vertical), dsmvc_gb::dev::Sample::u16,
                                     input, input_stride, output, output_stride,
                                     to_conversion(conversion), horizontal->plan, vertical->plan);
    });
}

int dsmvc_gb_inverse_2d_planes(dsmvc_gb_executor *executor, const dsmvc_gb_host_plane *planes, int32_t count) {
    return guarded([&] {
        if (count < 0 || (count > 0 && !planes)) throw std::invalid_argument("invalid plane list");
        std::vector<dsmvc_gb::HostPlane> list(static_cast<std::size_t>(count));
        for (int32_t i = 0; i < count; ++i) {
            const auto &p = planes[i];
            if (!p.horizontal || !p.vertical) throw std::invalid_argument("plane without plans");
            if (p.sample < DSMVC_GB_FLOAT32 || p.sample > DSMVC_GB_UINT16)
                throw std::invalid_argument("sample kind is invalid");
            auto &d = list[static_cast<std::size_t>(i)];
            d.horizontal = p.horizontal->plan.get();
            d.vertical = p.vertical->plan.get();
            d.horizontal_keep = p.horizontal->plan;
            d.vertical_keep = p.vertical->plan;
            d.sample = static_cast<dsmvc_gb::dev::Sample>(p.sample);
            d.input = p.input;
            d.input_stride = p.input_stride;
            d.output = p.output;
            d.output_stride = p.output_stride;
            d.conversion = p.sample == DSMVC_GB_FLOAT32 ? dsmvc_gb::IntegerConversion{} : to_conversion(&p.conversion);
        }
        exec_of(executor).inverse_2d_planes(list);
    });
}

namespace {

std::vector<dsmvc_gb::PlaneTask> task_list(const dsmvc_gb_plane_task *tasks, int32_t count) {
    if (count < 0 || (count > 0 && !tasks)) throw std::invalid_argument("invalid task list");
    std::vector<dsmvc_gb::PlaneTask> list(static_cast<std::size_t>(count));
    for (int32_t i = 0; i < count; ++i) {
        const auto &t = tasks[i];
        if (t.sample < DSMVC_GB_FLOAT32 || t.sample > DSMVC_GB_UINT16)
            throw std::invalid_argument("sample kind is invalid");
        auto &d = list[static_cast<std::size_t>(i)];
        d.horizontal = t.horizontal ? &plan_of(t.horizontal) : nullptr;
        d.vertical = t.vertical ? &plan_of(t.vertical) : nullptr;
        if (t.horizontal) d.horizontal_keep = t.horizontal->plan;
        if (t.vertical) d.vertical_keep = t.vertical->plan;
        d.input = t.input;
        d.input_stride = t.input_stride;
        d.output = t.output;
        d.output_stride = t.output_stride;
        d.sample = static_cast<dsmvc_gb::dev::Sample>(t.sample);
        d.vectors = t.vectors;
        d.conversion = to_conversion(&t.conversion);
    }
    return list;
}

} // namespace

int dsmvc_gb_run_batch(dsmvc_gb_executor *executor, const dsmvc_gb_plane_task *tasks, int32_t count,
                       void *stream, int32_t synchronize) {
    return guarded([&] { exec_of(executor).run_batch(task_list(tasks, count), stream, synchronize != 0); });
}

struct dsmvc_gb_batch {
    std::unique_ptr<dsmvc_gb::PreparedBatch> batch;
};

int dsmvc_gb_batch_create(dsmvc_gb_executor *executor, const dsmvc_gb_plane_task *tasks, int32_t count,
                          dsmvc_gb_batch **out) {
    return guarded([&] {
        if (!out) throw std::invalid_argument("output pointer is null");
        *out = nullptr;
        auto b = std::make_unique<dsmvc_gb_batch>();
        b->batch = exec_of(executor).prepare_batch(task_list(tasks, count));
        *out = b.release();
    });
}

int dsmvc_gb_batch_create_parts(dsmvc_gb_executor *executor, const dsmvc_gb_plane_task *tasks, int32_t count,
                                int32_t parts, dsmvc_gb_batch **out) {
    return guarded([&] {
        if (!out) throw std::invalid_argument("output pointer is null");
        *out = nullptr;
        auto b = std::make_unique<dsmvc_gb_batch>();
        b->batch = exec_of(executor).prepare_batch(task_list(tasks, count), nullptr, nullptr, 0, 0, parts);
        *out = b.release();
    });
}

int dsmvc_gb_batch_parts(const dsmvc_gb_batch *batch, int32_t *parts) {
    return guarded([&] {
        if (!batch || !parts) throw std::invalid_argument("batch or output is null");
        *parts = static_cast<int32_t>(batch->batch->parts());
    });
}

int dsmvc_gb_batch_launch(dsmvc_gb_batch *batch, void *stream) {
    return guarded([&] {
        if (!batch) throw std::invalid_argument("batch is null");
        batch->batch->launch(stream);
    });
}

int dsmvc_gb_batch_check(dsmvc_gb_batch *batch, void *stream) {
    return guarded([&] {
        if (!batch) throw std::invalid_argument("batch is null");
        batch->batch->check_status(stream);
    });
}

int dsmvc_gb_batch_info(const dsmvc_gb_batch *batch, int64_t *kernel_launches, int64_t *scratch_bytes,
                        int64_t *table_bytes) {
    return guarded([&] {
        if (!batch) throw std::invalid_argument("batch is null");
        if (kernel_launches) *kernel_launches = static_cast<int64_t>(batch->batch->kernel_launches());
        if (scratch_bytes) *scratch_bytes = static_cast<int64_t>(batch->batch->scratch_bytes());
        if (table_bytes) *table_bytes = static_cast<int64_t>(batch->batch->table_bytes());
    });
}

void dsmvc_gb_batch_destroy(dsmvc_gb_batch *batch) { delete batch; }

int dsmvc_gb_stream_check(dsmvc_gb_executor *executor, void *stream) {
    return guarded([&] { exec_of(executor).check_status(stream); });
}

int dsmvc_gb_stream_release(dsmvc_gb_executor *executor, void *stream) {
    return guarded([&] { exec_of(executor).release_stream(stream); });
}

int dsmvc_gb_inverse_2d_noalloc(const dsmvc_gb_plan *horizontal, const dsmvc_gb_plan *vertical,
                                int32_t sample, const void *input, int64_t input_stride,
                                void *output, int64_t output_stride,
                                const dsmvc_gb_conversion *conversion, void *stream) {
    return guarded([&] {
        if (sample < DSMVC_GB_FLOAT32 || sample > DSMVC_GB_UINT16)
            throw std::invalid_argument("sample kind is invalid");
        dsmvc_gb::dev::Conversion conv{0.0F, 1.0F, 1.0F, 0.0F, 255U};
        if (sample != DSMVC_GB_FLOAT32) {
            const auto c = to_conversion(conversion);
            conv = {c.input_offset, c.input_scale, c.output_scale, c.output_offset, c.output_maximum};
        }
        dsmvc_gb::inverse_2d_noalloc(plan_of(horizontal), plan_of(vertical),
                                     static_cast<dsmvc_gb::dev::Sample>(sample), input, input_stride,
                                     output, output_stride, conv, stream);
    });
}

int dsmvc_gb_measure_fp64_peak(int32_t device, double *tflops) {
    return guarded([&] {
        if (!tflops) throw std::invalid_argument("output is null");
        const int rc = dsmvc_gb::measure_fp64_peak(device, tflops);
        if (rc != 0)
            throw std::runtime_error(std::string("CUDA measuring the FP64 peak: ")
                                     + cudaGetErrorString(static_cast<cudaError_t>(rc)));
    });
}

int dsmvc_gb_profile(dsmvc_gb_executor *executor, int32_t enable) {
    return guarded([&] { exec_of(executor).set_profiling(enable != 0); });
}

int dsmvc_gb_profile_read(dsmvc_gb_executor *executor, dsmvc_gb_kernel_time *out,
                          int32_t capacity, int32_t *count) {
    return guarded([&] {
        if (!count || capacity < 0 || (capacity > 0 && !out))
            throw std::invalid_argument("invalid profile buffer");
        const auto times = exec_of(executor).kernel_times();
        *count = static_cast<int32_t>(times.size());
        for (std::size_t i = 0; i < times.size() && static_cast<int32_t>(i) < capacity; ++i) {
            auto &o = out[i];
            std::snprintf(o.name, sizeof(o.name), "%s", times[i].name.c_str());
            o.launches = times[i].launches;
            o.milliseconds = times[i].milliseconds;
            o.bytes = times[i].bytes;
        }
    });
}

struct dsmvc_gb_sweep {
    std::unique_ptr<dsmvc_gb::Sweep> sweep;
};

int dsmvc_gb_sweep_create(dsmvc_gb_executor *executor, const dsmvc_gb_plan *const *horizontal,
                          const dsmvc_gb_plan *const *vertical, int32_t count, const float *frame,
                          int64_t frame_stride, const dsmvc_gb_sweep_options *options, dsmvc_gb_sweep **out) {
    return guarded([&] {
        if (!out) throw std::invalid_argument("output handle is null");
        *out = nullptr;
        if (count <= 0 || !horizontal || !vertical) throw std::invalid_argument("invalid candidate list");
        auto s = std::make_unique<dsmvc_gb_sweep>();
        std::vector<dsmvc_gb::Sweep::Candidate> list;
        for (int32_t i = 0; i < count; ++i) {
            if (!horizontal[i] || !vertical[i]) throw std::invalid_argument("candidate plan is null");
            list.emplace_back(horizontal[i]->plan, vertical[i]->plan);
        }
        dsmvc_gb::SweepOptions o;
        if (options) {
            if (options->memory_budget < 0) throw std::invalid_argument("negative memory budget");
            o.memory_budget = static_cast<std::size_t>(options->memory_budget);
            o.autotune = options->autotune != 0;
            o.graph = options->graph != 0;
            o.fused_scoring = options->fused_scoring != 0;
        }
        s->sweep = std::make_unique<dsmvc_gb::Sweep>(exec_of(executor), list, frame, frame_stride, o);
        *out = s.release();
    });
}

int dsmvc_gb_sweep_run(dsmvc_gb_sweep *sweep, void *stream) {
    return guarded([&] {
        if (!sweep) throw std::invalid_argument("sweep is null");
        sweep->sweep->run(stream);
    });
}

int dsmvc_gb_sweep_run_plain(dsmvc_gb_sweep *sweep, void *stream) {
    return guarded([&] {
        if (!sweep) throw std::invalid_argument("sweep is null");
        sweep->sweep->run_plain(stream);
    });
}

int dsmvc_gb_sweep_scores(dsmvc_gb_sweep *sweep, float *scores, void *stream) {
    return guarded([&] {
        if (!sweep || !scores) throw std::invalid_argument("sweep or score buffer is null");
        sweep->sweep->read_scores(scores, stream);
    });
}

int dsmvc_gb_sweep_get_info(const dsmvc_gb_sweep *sweep, dsmvc_gb_sweep_info *out) {
    return guarded([&] {
        if (!sweep || !out) throw std::invalid_argument("sweep or output is null");
        const auto i = sweep->sweep->info();
        out->candidates = i.candidates;
        out->waves = i.waves;
        out->device_bytes = static_cast<int64_t>(i.device_bytes);
        out->kernel_launches = static_cast<int64_t>(i.kernel_launches);
        out->tune_milliseconds = i.tune_milliseconds;
        out->segment_rows = i.segment_rows;
        out->tuned_groups = static_cast<int32_t>(i.tuning.size());
        out->vectors_per_warp = i.vectors_per_warp;
        out->fused_candidates = i.fused_candidates;
    });
}

int dsmvc_gb_sweep_profile(dsmvc_gb_sweep *sweep, void *stream, double *milliseconds) {
    return guarded([&] {
        if (!sweep || !milliseconds) throw std::invalid_argument("sweep or output is null");
        const auto t = sweep->sweep->stage_milliseconds(stream);
        std::copy(t.begin(), t.end(), milliseconds);
    });
}

void dsmvc_gb_sweep_destroy(dsmvc_gb_sweep *sweep) { delete sweep; }

struct dsmvc_gb_server {
    std::unique_ptr<dsmvc_gb::Server> server;
};

int dsmvc_gb_server_create(dsmvc_gb_executor *executor, const dsmvc_gb_server_options *options,
                           dsmvc_gb_server **out) {
    return guarded([&] {
        if (!out) throw std::invalid_argument("output handle is null");
        *out = nullptr;
        dsmvc_gb::ServerOptions o;
        if (options) {
            if (options->memory_budget < 0) throw std::invalid_argument("negative memory budget");
            o.memory_budget = static_cast<std::size_t>(options->memory_budget);
            o.streams = options->streams;
            o.max_batch = options->max_batch;
        }
        auto s = std::make_unique<dsmvc_gb_server>();
        s->server = std::make_unique<dsmvc_gb::Server>(exec_of(executor), o);
        *out = s.release();
    });
}

int dsmvc_gb_server_submit(dsmvc_gb_server *server, const dsmvc_gb_host_plane *planes, int32_t count,
                           uint64_t *ticket) {
    return guarded([&] {
        if (!server || !ticket || count <= 0 || !planes) throw std::invalid_argument("invalid request");
        std::vector<dsmvc_gb::ServePlane> list(static_cast<std::size_t>(count));
        for (int32_t i = 0; i < count; ++i) {
            const auto &p = planes[i];
            if (!p.horizontal || !p.vertical) throw std::invalid_argument("request plane without plans");
            if (p.sample < DSMVC_GB_FLOAT32 || p.sample > DSMVC_GB_UINT16)
                throw std::invalid_argument("sample kind is invalid");
            auto &d = list[static_cast<std::size_t>(i)];
            d.horizontal = p.horizontal->plan;
            d.vertical = p.vertical->plan;
            d.input = p.input;
            d.input_stride = p.input_stride;
            d.output = p.output;
            d.output_stride = p.output_stride;
            d.sample = static_cast<dsmvc_gb::dev::Sample>(p.sample);
            d.conversion = p.sample == DSMVC_GB_FLOAT32 ? dsmvc_gb::IntegerConversion{} : to_conversion(&p.conversion);
        }
        *ticket = server->server->submit(std::move(list));
    });
}

int dsmvc_gb_server_wait(dsmvc_gb_server *server, uint64_t ticket) {
    int status = DSMVC_GB_OK;
    std::string message;
    const int rc = guarded([&] {
        if (!server) throw std::invalid_argument("server is null");
        status = server->server->wait(ticket, &message);
    });
    if (rc != DSMVC_GB_OK) return rc;
    g_error = message;
    return status;
}

int dsmvc_gb_server_poll(dsmvc_gb_server *server, uint64_t ticket, int32_t *done) {
    return guarded([&] {
        if (!server || !done) throw std::invalid_argument("server or output is null");
        *done = server->server->done(ticket) ? 1 : 0;
    });
}

int dsmvc_gb_server_get_stats(dsmvc_gb_server *server, dsmvc_gb_server_stats *out) {
    return guarded([&] {
        if (!server || !out) throw std::invalid_argument("server or output is null");
        const auto s = server->server->stats();
        out->submitted = s.submitted;
        out->completed = s.completed;
        out->failed = s.failed;
        out->batches = s.batches;
        out->latency_p50_ms = s.latency_p50_ms;
        out->latency_p99_ms = s.latency_p99_ms;
        out->latency_mean_ms = s.latency_mean_ms;
        out->latency_max_ms = s.latency_max_ms;
        out->peak_device_bytes = static_cast<int64_t>(s.peak_device_bytes);
        out->source_pixels = s.source_pixels;
        out->mean_batch_requests = s.mean_batch_requests;
    });
}

int dsmvc_gb_server_reset_stats(dsmvc_gb_server *server) {
    return guarded([&] {
        if (!server) throw std::invalid_argument("server is null");
        server->server->reset_stats();
    });
}

void dsmvc_gb_server_destroy(dsmvc_gb_server *server) { delete server; }

} // extern "C"

namespace {

// Fake registrations for the registry's tests (no page-locking).
dsmvc_gb::BlockRegistration fake_owned(void *, std::size_t) { return dsmvc_gb::BlockRegistration::owned; }
dsmvc_gb::BlockRegistration fake_foreign(void *, std::size_t) { return dsmvc_gb::BlockRegistration::foreign; }
dsmvc_gb::BlockRegistration fake_failed(void *, std::size_t) { return dsmvc_gb::BlockRegistration::failed; }
void fake_unregister(void *, std::size_t) {}

} // namespace

extern "C" {

int dsmvc_gb_host_blocks_set_limit(const void *owner, int64_t bytes) {
    return guarded([&] {
        if (bytes < 0) throw std::invalid_argument("negative limit");
        dsmvc_gb::host_blocks::set_limit(owner, static_cast<std::size_t>(bytes));
    });
}

int dsmvc_gb_host_blocks_note_use(const void *owner, void *base, int64_t size) {
    return guarded([&] {
        if (size < 0) throw std::invalid_argument("negative block size");
        dsmvc_gb::host_blocks::note_use(owner, base, static_cast<std::size_t>(size));
    });
}

int dsmvc_gb_host_blocks_covered(const void *pointer, int64_t bytes, int32_t *covered) {
    return guarded([&] {
        if (!covered || bytes < 0) throw std::invalid_argument("invalid range or null output");
        *covered = dsmvc_gb::host_blocks::covered(pointer, static_cast<std::size_t>(bytes)) ? 1 : 0;
    });
}

int dsmvc_gb_host_blocks_release(void *base, int64_t size) {
    return guarded([&] {
        if (size < 0) throw std::invalid_argument("negative block size");
        dsmvc_gb::host_blocks::release_block(base, static_cast<std::size_t>(size));
    });
}

int dsmvc_gb_host_blocks_drop_owner(const void *owner) {
    return guarded([&] { dsmvc_gb::host_blocks::drop_owner(owner); });
}

int dsmvc_gb_host_blocks_get_stats(dsmvc_gb_host_block_stats *out) {
    return guarded([&] {
        if (!out) throw std::invalid_argument("output is null");
        const auto s = dsmvc_gb::host_blocks::stats();
        out->registrations = s.registrations;
        out->failures = s.failures;
        out->cap_refusals = s.cap_refusals;
        out->hits = s.hits;
        out->misses = s.misses;
        out->released = s.released;
        out->registered_bytes = s.registered_bytes;
        out->peak_bytes = s.peak_bytes;
    });
}

int dsmvc_gb_host_blocks_test_registrar(int32_t mode) {
    return guarded([&] {
        using dsmvc_gb::BlockRegistrar;
        switch (mode) {
        case 0: dsmvc_gb::host_blocks::set_registrar(BlockRegistrar{}); break;
        case 1: dsmvc_gb::host_blocks::set_registrar(BlockRegistrar{fake_owned, fake_unregister}); break;
        case 2: dsmvc_gb::host_blocks::set_registrar(BlockRegistrar{fake_foreign, fake_unregister}); break;
        case 3: dsmvc_gb::host_blocks::set_registrar(BlockRegistrar{fake_failed, fake_unregister}); break;
        default: throw std::invalid_argument("registrar mode must be 0..3");
        }
    });
}

int dsmvc_gb_host_register(void *base, int64_t size, int32_t *outcome) {
    return guarded([&] {
        if (!base || size <= 0 || !outcome) throw std::invalid_argument("invalid block or null output");
        *outcome = static_cast<int32_t>(dsmvc_gb::host_blocks::cuda_register(base, static_cast<std::size_t>(size)));
    });
}

int dsmvc_gb_host_unregister(void *base) {
    return guarded([&] {
        if (!base) throw std::invalid_argument("block is null");
        dsmvc_gb::host_blocks::cuda_unregister(base, 0);
    });
}

} // extern "C"
