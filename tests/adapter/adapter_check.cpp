// Test driver for the drop-in backend (adapter/gb300_cuda_executor.*),
// compiled against the reference's include/dsmvc/engine.hpp and linked with
// the reference engine (oracle/_ref) and libdsmvc_gb300.so by
// tests/test_adapter.py.
//
//   adapter_check plans   plans built by the reference planner import
//                         bit-identical to the GB300 planner's own; invalid
//                         plans are refused (no GPU needed)
//   adapter_check gpu     the reference plans run through the adapter class
//                         (prepared and unprepared) give the GB300 executor's
//                         own results bit for bit
//   adapter_check random [N]  N seeded random requests: the reference planner
//                         and the GB300 planner agree bit for bit (no GPU)
//   adapter_check blocks  the adapter's registrar in the engine's host block
//                         registry page-locks a frame-pool block reported
//                         twice (none with DSMVC_CUDA_DIRECT_IO=0)
#include "gb300_cuda_executor.hpp"

#include "dsmvc_gb300.h"

#include <dsmvc/engine.hpp>
#include <dsmvc/host_blocks.hpp>

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <memory>
#include <random>
#include <stdexcept>
#include <string>
#include <vector>

namespace {

int failures = 0;

void expect(bool ok, const std::string &what) {
    if (!ok) {
        std::printf("FAIL %s\n", what.c_str());
        ++failures;
    }
}

struct Case {
    dsmvc::AxisRequest ref;
    dsmvc_gb_axis_request own;
};

Case make_case(int src, int dst, double active, double shift, int kind, int taps, double b, double c,
               double blur, int border, int f64) {
    Case k{};
    k.ref.source_size = src;
    k.ref.destination_size = dst;
    k.ref.active_length = active;
    k.ref.shift = shift;
    k.ref.kernel.kind = static_cast<dsmvc::KernelKind>(kind);
    k.ref.kernel.taps = taps;
    k.ref.kernel.b = b;
    k.ref.kernel.c = c;
    k.ref.kernel.blur = blur;
    k.ref.border = static_cast<dsmvc::BorderMode>(border);
    k.ref.f64_mode = static_cast<dsmvc::F64Mode>(f64);
    k.own = {src, dst, active, shift, kind, taps, b, c, blur, border, f64};
    return k;
}

std::vector<Case> cases() {
    return {
        make_case(1920, 1440, 1440.0, 0.0, DSMVC_GB_LANCZOS, 3, 0, 0.5, 1.0, DSMVC_GB_REPEAT, 0),
        make_case(1080, 810, 810.0, 0.0, DSMVC_GB_LANCZOS, 3, 0, 0.5, 1.0, DSMVC_GB_REPEAT, 0),
        make_case(960, 720, 720.0, 0.0625, DSMVC_GB_LANCZOS, 3, 0, 0.5, 1.0, DSMVC_GB_REPEAT, 0),
        make_case(640, 427, 426.5, 0.2, DSMVC_GB_BICUBIC, 3, 1.0 / 3.0, 1.0 / 3.0, 1.1, DSMVC_GB_MIRROR, 0),
        make_case(384, 256, 256.0, 0.0, DSMVC_GB_SPLINE64, 3, 0, 0.5, 1.1, DSMVC_GB_SYMMETRIC, 2),
        make_case(216, 144, 144.0, 0.0, DSMVC_GB_SPLINE64, 3, 0, 0.5, 1.1, DSMVC_GB_SYMMETRIC, 2),
        // Ill-conditioned: automatic mode keeps Float64.
        make_case(1080, 980, 978.1, 0.95, DSMVC_GB_LANCZOS, 2, 0, 0.5, 1.0, DSMVC_GB_SYMMETRIC, 0),
        make_case(300, 200, 200.0, 0.0, DSMVC_GB_BILINEAR, 3, 0, 0.5, 1.0, DSMVC_GB_ZERO, 1),
    };
}

template <class T>
bool same_array(const dsmvc_gb_plan *a, const dsmvc_gb_plan *b, int which) {
    const void *pa = nullptr, *pb = nullptr;
    std::uint64_t na = 0, nb = 0;
    if (dsmvc_gb_plan_get_array(a, which, &pa, &na) || dsmvc_gb_plan_get_array(b, which, &pb, &nb))
        return false;
    return na == nb && (na == 0 || std::memcmp(pa, pb, na * sizeof(T)) == 0);
}

// The reference planner's plan of `k`, imported, against the GB300 planner's
// own plan of the same request: scalars, all ten arrays and both plan hashes.
void compare_plan(const Case &k) {
    {
        const auto ref = dsmvc::build_axis_plan(k.ref);
        auto *imported = static_cast<dsmvc_gb_plan *>(dsmvc::gb300_detail::Gb300Executor::import_plan(ref));
        dsmvc_gb_plan *own = nullptr;
        expect(dsmvc_gb_plan_build(&k.own, nullptr, nullptr, &own) == DSMVC_GB_OK, "own plan builds");
        dsmvc_gb_plan_info ia{}, io{};
        dsmvc_gb_plan_get_info(imported, &ia);
        dsmvc_gb_plan_get_info(own, &io);
        const std::string tag = std::to_string(k.own.source_size) + "->" + std::to_string(k.own.destination_size);
        expect(ia.source_size == io.source_size && ia.destination_size == io.destination_size
                   && ia.support == io.support && ia.half_bandwidth == io.half_bandwidth
                   && ia.requires_float64 == io.requires_float64 && ia.max_row_entries == io.max_row_entries
                   && ia.normal_rcond == io.normal_rcond && ia.normal_inf_norm == io.normal_inf_norm
                   && ia.requires_float64 == (ref.requires_float64() ? 1 : 0),
               "plan scalars " + tag);
        expect(same_array<std::uint32_t>(imported, own, 0) && same_array<std::int32_t>(imported, own, 1)
                   && same_array<float>(imported, own, 2) && same_array<float>(imported, own, 3)
                   && same_array<float>(imported, own, 4) && same_array<float>(imported, own, 5)
                   && same_array<double>(imported, own, 6) && same_array<double>(imported, own, 7)
                   && same_array<double>(imported, own, 8) && same_array<double>(imported, own, 9),
               "plan arrays " + tag);
        // An imported plan carries no request: hashes need one.
        std::uint64_t f = 0, c = 0, fo = 0, co = 0;
        expect(dsmvc_gb_plan_hashes(imported, nullptr, &f, &c) == DSMVC_GB_INVALID_ARGUMENT,
               "hashes without request refused " + tag);
        expect(dsmvc_gb_plan_hashes(imported, &k.own, &f, &c) == DSMVC_GB_OK
                   && dsmvc_gb_plan_hashes(own, nullptr, &fo, &co) == DSMVC_GB_OK && f == fo && c == co,
               "plan hashes " + tag);
        dsmvc_gb_plan_release(imported);
        dsmvc_gb_plan_release(own);
    }
}

void check_plans() {
    int checked = 0;
    for (const auto &k : cases()) {
        compare_plan(k);
        ++checked;
    }
    // Invalid plans are refused like AxisPlan::check_valid refuses them.
    const auto good = dsmvc::build_axis_plan(cases()[3].ref);
    auto refused = [&](dsmvc::AxisPlan bad, const char *what) {
        try {
            dsmvc_gb_plan_release(
                static_cast<dsmvc_gb_plan *>(dsmvc::gb300_detail::Gb300Executor::import_plan(bad)));
            expect(false, std::string("refused: ") + what);
        } catch (const std::invalid_argument &) {
        }
    };
    auto bad = good;
    bad.transpose_weights[5] = std::numeric_limits<float>::quiet_NaN();
    refused(bad, "non-finite weight");
    bad = good;
    std::swap(bad.transpose_indices[0], bad.transpose_indices[1]);
    refused(bad, "descending indices");
    bad = good;
    bad.lower_ld.pop_back();
    refused(bad, "short factor array");
    bad = good;
    bad.half_bandwidth = bad.destination_size;
    refused(bad, "half-bandwidth beyond the destination");
    bad = good;
    bad.normal_bands_f64.assign(good.inverse_diagonal.size(), 1.0);
    refused(bad, "partial Float64 arrays");
    bad = good;
    bad.transpose_offsets.back() += 1;
    refused(bad, "offsets past the entries");
    std::printf("plans ok: %d imported bit-identical, 6 invalid plans refused\n", checked);
}

std::vector<std::uint16_t> frame_u16(int w, int h, unsigned seed) {
    std::mt19937 rng(seed);
    std::uniform_int_distribution<int> d(4096, 60160);
    std::vector<std::uint16_t> v(static_cast<std::size_t>(w) * h);
    for (auto &x : v) x = static_cast<std::uint16_t>(d(rng));
    return v;
}

std::vector<float> frame_f32(int w, int h, unsigned seed) {
    std::mt19937 rng(seed);
    std::uniform_real_distribution<float> d(0.0F, 1.0F);
    std::vector<float> v(static_cast<std::size_t>(w) * h);
    for (auto &x : v) x = d(rng);
    return v;
}

void check_gpu() {
    const auto all = cases();
    dsmvc::gb300_detail::Gb300Executor adapter;
    dsmvc_gb_executor *ex = nullptr;
    expect(dsmvc_gb_executor_create(0, &ex) == DSMVC_GB_OK, "own executor");
    auto own_plan = [](const Case &k) {
        dsmvc_gb_plan *p = nullptr;
        dsmvc_gb_plan_build(&k.own, nullptr, nullptr, &p);
        return p;
    };
    // Integer 2D (luma of the YUV420P16 workload): prepared plans.
    {
        auto h = std::make_shared<const dsmvc::AxisPlan>(dsmvc::build_axis_plan(all[0].ref));
        auto v = std::make_shared<const dsmvc::AxisPlan>(dsmvc::build_axis_plan(all[1].ref));
        adapter.prepare(h);
        adapter.prepare(v);
        adapter.seal();
        const auto x = frame_u16(1920, 1080, 7);
        std::vector<std::uint16_t> got(1440 * 810), want(1440 * 810);
        const dsmvc::IntegerConversion conv{4096.0F, 1.0F / 56064.0F, 56064.0F, 4096.0F, 65535U};
        adapter.inverse_2d_u16(*h, *v, x.data(), 1920, got.data(), 1440, conv, {});
        auto *oh = own_plan(all[0]);
        auto *ov = own_plan(all[1]);
        const dsmvc_gb_conversion c{conv.input_offset, conv.input_scale, conv.output_scale,
                                    conv.output_offset, conv.output_maximum};
        expect(dsmvc_gb_inverse_2d_u16(ex, oh, ov, x.data(), 1920, want.data(), 1440, &c) == DSMVC_GB_OK,
               "own u16 call");
        expect(got == want, "prepared u16 2D equals the executor's");
        dsmvc_gb_plan_release(oh);
        dsmvc_gb_plan_release(ov);
    }
    // Float32 2D with unprepared plans (imported for the call), and a
    // Float64 pair.
    for (int pair : {3, 4}) {
        const auto &hk = all[pair];
        const auto &vk = all[pair == 3 ? 3 : 5];
        const auto h = dsmvc::build_axis_plan(hk.ref);
        const auto v = dsmvc::build_axis_plan(vk.ref);
        const int sw = hk.own.source_size, sh = vk.own.source_size;
        const int dw = hk.own.destination_size, dh = vk.own.destination_size;
        const auto x = frame_f32(sw, sh, 11 + pair);
        std::vector<float> got(static_cast<std::size_t>(dw) * dh), want(got.size());
        adapter.inverse_2d(h, v, x.data(), sw, got.data(), dw, {});
        auto *oh = own_plan(hk);
        auto *ov = own_plan(vk);
        expect(dsmvc_gb_inverse_2d(ex, oh, ov, x.data(), sw, want.data(), dw) == DSMVC_GB_OK, "own 2D call");
        expect(std::memcmp(got.data(), want.data(), got.size() * sizeof(float)) == 0,
               "unprepared 2D equals the executor's (pair " + std::to_string(pair) + ")");
        // Rows only, unprepared.
        std::vector<float> rows(static_cast<std::size_t>(dw) * sh), rows_want(rows.size());
        adapter.inverse_rows(h, x.data(), sw, rows.data(), dw, sh, {});
        expect(dsmvc_gb_inverse_rows(ex, oh, x.data(), sw, rows_want.data(), dw, sh) == DSMVC_GB_OK,
               "own rows call");
        expect(std::memcmp(rows.data(), rows_want.data(), rows.size() * sizeof(float)) == 0,
               "unprepared rows equal the executor's");
        dsmvc_gb_plan_release(oh);
        dsmvc_gb_plan_release(ov);
    }
    // Errors arrive as the reference's exception types.
    try {
        const auto h = dsmvc::build_axis_plan(all[3].ref);
        std::vector<float> x(10), y(10);
        adapter.inverse_2d(h, h, x.data(), 1, y.data(), 1, {});
        expect(false, "short strides refused");
    } catch (const std::invalid_argument &) {
    }
    dsmvc_gb_executor_destroy(ex);
    std::printf("gpu ok\n");
}

// The engine's host block registry with the adapter's registrar installed:
// a frame-pool block reported twice is page-locked (registering it again
// finds it page-locked elsewhere), calls from and to it give the same bytes
// as from plain memory, and dropping its owner unregisters it.  With
// DSMVC_CUDA_DIRECT_IO=0 no registrar is installed and nothing is locked.
void check_blocks() {
    namespace hb = dsmvc::host_blocks;
    const char *direct = std::getenv("DSMVC_CUDA_DIRECT_IO");
    const bool installed = !(direct && std::string(direct) == "0") && !std::getenv("DSMVC_CUDA_HOST_TRANSFER");
    const auto all = cases();
    dsmvc::gb300_detail::Gb300Executor adapter;
    expect(hb::enabled(hb::Domain::cuda) == installed, "registrar installed as requested");
    const auto h = dsmvc::build_axis_plan(all[0].ref);
    const auto v = dsmvc::build_axis_plan(all[1].ref);
    const dsmvc::IntegerConversion conv{4096.0F, 1.0F / 56064.0F, 56064.0F, 4096.0F, 65535U};
    const auto x = frame_u16(1920, 1080, 5);
    std::vector<std::uint16_t> want(1440 * 810);
    adapter.inverse_2d_u16(h, v, x.data(), 1920, want.data(), 1440, conv, {});
    // One pool block holding a source frame and a destination frame.
    std::vector<std::uint16_t> pool(x.size() + want.size());
    const std::size_t bytes = pool.size() * sizeof(std::uint16_t);
    std::uint16_t *out = pool.data() + x.size();
    int token = 0;
    const void *owner = &token;
    hb::set_limit(owner, 64U << 20);
    const auto s0 = hb::stats(hb::Domain::cuda);
    for (int use = 0; use < 3; ++use) {
        std::memcpy(pool.data(), x.data(), x.size() * sizeof(std::uint16_t));
        std::memset(out, 0, want.size() * sizeof(std::uint16_t));
        hb::note_use(hb::Domain::cuda, owner, pool.data(), bytes);
        adapter.inverse_2d_u16(h, v, pool.data(), 1920, out, 1440, conv, {});
        expect(std::memcmp(out, want.data(), want.size() * sizeof(std::uint16_t)) == 0,
               "frames in the pool block descale alike (use " + std::to_string(use) + ")");
    }
    const auto s1 = hb::stats(hb::Domain::cuda);
    const bool leased = static_cast<bool>(hb::acquire(hb::Domain::cuda, pool.data(), bytes));
    std::int32_t outcome = -2;
    expect(dsmvc_gb_host_register(pool.data(), static_cast<std::int64_t>(bytes), &outcome) == DSMVC_GB_OK,
           "register call");
    if (installed) {
        expect(s1.registrations - s0.registrations == 1 && s1.failures == s0.failures, "one registration");
        expect(s1.registered_bytes - s0.registered_bytes == bytes, "registered bytes");
        expect(leased, "the block is leased");
        expect(outcome == 1, "the block is page-locked");
    } else {
        expect(s1.registrations == s0.registrations && !leased, "nothing registered");
        expect(outcome == 0, "the block is not page-locked");
        expect(dsmvc_gb_host_unregister(pool.data()) == DSMVC_GB_OK, "unregister call");
    }
    hb::drop_owner(owner);
    if (installed) {
        expect(hb::stats(hb::Domain::cuda).released - s1.released == 1, "dropping the owner releases");
        outcome = -2;
        expect(dsmvc_gb_host_register(pool.data(), static_cast<std::int64_t>(bytes), &outcome) == DSMVC_GB_OK &&
                   outcome == 0,
               "the block is unregistered");
        expect(dsmvc_gb_host_unregister(pool.data()) == DSMVC_GB_OK, "unregister call");
    }
    std::printf("blocks ok (%s)\n", installed ? "registrar installed" : "no registrar");
}

// Seeded random requests (every kernel, border and Float64 mode; shifts,
// active lengths and blur away from their defaults): the reference planner
// and the GB300 planner give bit-identical plans, or both refuse the request.
void check_random_plans(int count, unsigned seed) {
    std::mt19937 rng(seed);
    auto uniform = [&](double lo, double hi) { return std::uniform_real_distribution<double>(lo, hi)(rng); };
    auto pick = [&](int lo, int hi) { return std::uniform_int_distribution<int>(lo, hi)(rng); };
    const int kinds[] = {DSMVC_GB_BILINEAR, DSMVC_GB_BICUBIC, DSMVC_GB_LANCZOS,
                         DSMVC_GB_SPLINE16, DSMVC_GB_SPLINE36, DSMVC_GB_SPLINE64};
    int built = 0, refused = 0;
    for (int i = 0; i < count; ++i) {
        const int src = pick(9, 1200), dst = pick(8, src);
        double active = uniform(0.0, 1.0) < 0.5 ? dst - uniform(0.0, 2.0) : dst;
        if (active <= 0.0) active = dst;
        const Case k = make_case(src, dst, active, uniform(-1.0, 1.0), kinds[pick(0, 5)], pick(1, 5),
                                 uniform(0.0, 0.5), uniform(0.0, 0.6),
                                 uniform(0.0, 1.0) < 0.6 ? 1.0 : uniform(0.8, 1.6), pick(0, 4), pick(0, 2));
        bool ref_ok = true;
        try {
            (void)dsmvc::build_axis_plan(k.ref);
        } catch (const std::exception &) {
            ref_ok = false;
        }
        dsmvc_gb_plan *own = nullptr;
        const bool own_ok = dsmvc_gb_plan_build(&k.own, nullptr, nullptr, &own) == DSMVC_GB_OK;
        dsmvc_gb_plan_release(own);
        expect(ref_ok == own_ok, "both planners accept or refuse request " + std::to_string(i));
        if (ref_ok && own_ok) {
            compare_plan(k);
            ++built;
        } else {
            ++refused;
        }
    }
    std::printf("random plans ok: %d bit-identical, %d refused by both\n", built, refused);
}

} // namespace

int main(int argc, char **argv) {
    const std::string mode = argc > 1 ? argv[1] : "plans";
    try {
        if (mode == "plans") check_plans();
        else if (mode == "gpu") check_gpu();
        else if (mode == "blocks") check_blocks();
        else if (mode == "random") check_random_plans(argc > 2 ? std::atoi(argv[2]) : 300, 20261204U);
        else {
            std::printf("unknown mode %s\n", mode.c_str());
            return 2;
        }
    } catch (const std::exception &e) {
        std::printf("FAIL exception: %s\n", e.what());
        return 1;
    }
    return failures ? 1 : 0;
}
