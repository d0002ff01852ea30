// C-ABI shim over the reference's own CPU engine, compiled from the
// reference sources by oracle/ref/Makefile into oracle/_ref/.  Test
// infrastructure only: it lets tests/golden/make_golden.py and the CPU
// baseline call dsmvc::build_axis_plan and dsmvc::CpuExecutor
// (include/dsmvc/engine.hpp:180-293) through plain C entry points.
#include <dsmvc/engine.hpp>

#include <cstdint>
#include <cstring>
#include <exception>
#include <memory>
#include <stdexcept>

namespace {

struct RefRequest {
    std::int32_t source_size;
    std::int32_t destination_size;
    double active_length;
    double shift;
    std::int32_t kind;
    std::int32_t taps;
    double b;
    double c;
    double blur;
    std::int32_t border;
    std::int32_t f64_mode;
};

struct RefConversion {
    float input_offset;
    float input_scale;
    float output_scale;
    float output_offset;
    std::uint32_t output_maximum;
};

using Plan = std::shared_ptr<const dsmvc::AxisPlan>;

template <class F>
int guarded(F &&f) {
    try {
        f();
        return 0;
    } catch (const std::invalid_argument &) {
        return 1;
    } catch (const std::length_error &) {
        return 3;
    } catch (const std::out_of_range &) {
        return 3;
    } catch (const std::runtime_error &) {
        return 2;
    } catch (...) {
        return 2;
    }
}

dsmvc::CpuExecutor executor(int path) {
    return dsmvc::CpuExecutor(path == 0 ? dsmvc::CpuPath::scalar
                                        : dsmvc::CpuPath::automatic);
}

} // namespace

extern "C" {

int ref_plan_build(const RefRequest *r, void **out) {
    return guarded([&] {
        dsmvc::AxisRequest q;
        q.source_size = r->source_size;
        q.destination_size = r->destination_size;
        q.active_length = r->active_length;
        q.shift = r->shift;
        q.kernel.kind = static_cast<dsmvc::KernelKind>(r->kind);
        q.kernel.taps = r->taps;
        q.kernel.b = r->b;
        q.kernel.c = r->c;
        q.kernel.blur = r->blur;
        q.border = static_cast<dsmvc::BorderMode>(r->border);
        q.f64_mode = static_cast<dsmvc::F64Mode>(r->f64_mode);
        *out = new Plan(std::make_shared<const dsmvc::AxisPlan>(
            dsmvc::build_axis_plan(q)));
    });
}

void ref_plan_free(void *plan) { delete static_cast<Plan *>(plan); }

// which: 0 offsets(u32) 1 indices(i32) 2 weights(f32) 3 lower_ld 4 upper_l
// 5 inverse_diagonal 6 weights_f64 7 normal_bands_f64 8 ldlt_bands_f64
// 9 inverse_diagonal_f64.  Returns the element count and the data pointer.
std::size_t ref_plan_array(const void *plan, int which, const void **data) {
    const auto &p = **static_cast<const Plan *>(plan);
    switch (which) {
    case 0: *data = p.transpose_offsets.data(); return p.transpose_offsets.size();
    case 1: *data = p.transpose_indices.data(); return p.transpose_indices.size();
    case 2: *data = p.transpose_weights.data(); return p.transpose_weights.size();
    case 3: *data = p.lower_ld.data(); return p.lower_ld.size();
    case 4: *data = p.upper_l.data(); return p.upper_l.size();
    case 5: *data = p.inverse_diagonal.data(); return p.inverse_diagonal.size();
    case 6: *data = p.transpose_weights_f64.data(); return p.transpose_weights_f64.size();
    case 7: *data = p.normal_bands_f64.data(); return p.normal_bands_f64.size();
    case 8: *data = p.ldlt_bands_f64.data(); return p.ldlt_bands_f64.size();
    case 9: *data = p.inverse_diagonal_f64.data(); return p.inverse_diagonal_f64.size();
    }
    *data = nullptr;
    return 0;
}

// out: source, destination, support, half_bandwidth, requires_f64
void ref_plan_ints(const void *plan, std::int32_t *out) {
    const auto &p = **static_cast<const Plan *>(plan);
    out[0] = p.source_size;
    out[1] = p.destination_size;
    out[2] = p.support;
    out[3] = p.half_bandwidth;
    out[4] = p.requires_float64() ? 1 : 0;
}

double ref_plan_rcond(const void *plan) {
    return (*static_cast<const Plan *>(plan))->normal_rcond;
}

int ref_inverse_rows(int path, const void *plan, const float *in,
                     std::ptrdiff_t is, float *out, std::ptrdiff_t os,
                     std::int32_t rows) {
    return guarded([&] {
        executor(path).inverse_rows(**static_cast<const Plan *>(plan), in, is,
                                    out, os, rows);
    });
}

int ref_inverse_columns(int path, const void *plan, const float *in,
                        std::ptrdiff_t is, float *out, std::ptrdiff_t os,
                        std::int32_t columns) {
    return guarded([&] {
        executor(path).inverse_columns(**static_cast<const Plan *>(plan), in,
                                       is, out, os, columns);
    });
}

int ref_inverse_2d(int path, const void *h, const void *v, const float *in,
                   std::ptrdiff_t is, float *out, std::ptrdiff_t os) {
    return guarded([&] {
        executor(path).inverse_2d(**static_cast<const Plan *>(h),
                                  **static_cast<const Plan *>(v), in, is,
                                  out, os);
    });
}

int ref_inverse_2d_u8(int path, const void *h, const void *v,
                      const std::uint8_t *in, std::ptrdiff_t is,
                      std::uint8_t *out, std::ptrdiff_t os,
                      const RefConversion *c) {
    return guarded([&] {
        const dsmvc::IntegerConversion conv{c->input_offset, c->input_scale,
                                            c->output_scale, c->output_offset,
                                            c->output_maximum};
        executor(path).inverse_2d_u8(**static_cast<const Plan *>(h),
                                     **static_cast<const Plan *>(v), in, is,
                                     out, os, conv);
    });
}

int ref_inverse_2d_u16(int path, const void *h, const void *v,
                       const std::uint16_t *in, std::ptrdiff_t is,
                       std::uint16_t *out, std::ptrdiff_t os,
                       const RefConversion *c) {
    return guarded([&] {
        const dsmvc::IntegerConversion conv{c->input_offset, c->input_scale,
                                            c->output_scale, c->output_offset,
                                            c->output_maximum};
        executor(path).inverse_2d_u16(**static_cast<const Plan *>(h),
                                      **static_cast<const Plan *>(v), in, is,
                                      out, os, conv);
    });
}

} // extern "C"
