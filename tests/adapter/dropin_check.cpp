// The reference engine with the GB300 backend switched in the way a
// maintainer does it (the CUDA executor's include and type, the two device
// probes): the reference's own src/executor.cpp and src/backend.cpp, built
// by tests/test_dropin_engine.py with their CUDA backend replaced by
// adapter/gb300_cuda_executor.*, driven through the reference's public API
// (include/dsmvc/engine.hpp) only.
//
//   dropin_check caps   the capability table lists the CUDA backend as
//                       compiled, available exactly when a GPU is; without
//                       a GPU, Executor(BackendKind::cuda) is refused
//   dropin_check gpu    dsmvc::Executor(BackendKind::cuda) runs the Delanczos
//                       1080p -> 810p luma descale of prepared plans: within
//                       1 code of Executor(BackendKind::cpu, CpuPath::scalar)
//                       and bit-identical to the GB300 C ABI's own call
#include "dsmvc_gb300.h"

#include <dsmvc/engine.hpp>

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
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

dsmvc::AxisRequest lanczos3(int src, int dst) {
    dsmvc::AxisRequest r;
    r.source_size = src;
    r.destination_size = dst;
    r.active_length = dst;
    r.shift = 0.0;
    r.kernel.kind = dsmvc::KernelKind::lanczos;
    r.kernel.taps = 3;
    r.border = dsmvc::BorderMode::repeat;
    return r;
}

void check_caps() {
    const bool gpu = dsmvc_gb_cuda_available() != 0;
    bool listed = false;
    for (const auto &c : dsmvc::backend_capabilities()) {
        if (c.kind != dsmvc::BackendKind::cuda) continue;
        listed = true;
        expect(c.compiled, "CUDA backend compiled");
        expect(c.device_available == gpu, "CUDA availability follows the GB300 library");
    }
    expect(listed, "CUDA backend listed");
    expect(dsmvc::cuda_compiled() && dsmvc::cuda_available() == gpu, "cuda_compiled / cuda_available");
    if (!gpu) {
        bool refused = false;
        try {
            dsmvc::Executor ex(dsmvc::BackendKind::cuda);
        } catch (const std::exception &) {
            refused = true;
        }
        expect(refused, "Executor(cuda) refused without a GPU");
    }
    std::printf("caps ok (gpu %s)\n", gpu ? "present" : "absent");
}

void check_gpu() {
    const auto h = std::make_shared<const dsmvc::AxisPlan>(dsmvc::build_axis_plan(lanczos3(1920, 1440)));
    const auto v = std::make_shared<const dsmvc::AxisPlan>(dsmvc::build_axis_plan(lanczos3(1080, 810)));
    dsmvc::Executor gpu(dsmvc::BackendKind::cuda);
    expect(gpu.backend() == dsmvc::BackendKind::cuda && std::string(gpu.name()) == "cuda", "CUDA executor");
    gpu.prepare(h);
    gpu.prepare(v);
    gpu.seal();
    std::mt19937 rng(9);
    std::uniform_int_distribution<int> d(4096, 60160);
    std::vector<std::uint16_t> x(1920 * 1080);
    for (auto &s : x) s = static_cast<std::uint16_t>(d(rng));
    const dsmvc::IntegerConversion conv{4096.0F, 1.0F / 56064.0F, 56064.0F, 4096.0F, 65535U};
    std::vector<std::uint16_t> got(1440 * 810), cpu(1440 * 810), own(1440 * 810);
    gpu.inverse_2d_u16(*h, *v, x.data(), 1920, got.data(), 1440, conv);
    dsmvc::Executor scalar(dsmvc::BackendKind::cpu, dsmvc::CpuPath::scalar);
    scalar.inverse_2d_u16(*h, *v, x.data(), 1920, cpu.data(), 1440, conv);
    int worst = 0;
    for (std::size_t i = 0; i < got.size(); ++i) worst = std::max(worst, std::abs(int(got[i]) - int(cpu[i])));
    expect(worst <= 1, "within 1 code of the CPU scalar route (" + std::to_string(worst) + ")");
    // The same request through the GB300 C ABI directly.
    dsmvc_gb_executor *ex = nullptr;
    dsmvc_gb_plan *oh = nullptr, *ov = nullptr;
    const dsmvc_gb_axis_request rh{1920, 1440, 1440.0, 0.0, DSMVC_GB_LANCZOS, 3, 0.0, 0.5, 1.0, DSMVC_GB_REPEAT, 0};
    const dsmvc_gb_axis_request rv{1080, 810, 810.0, 0.0, DSMVC_GB_LANCZOS, 3, 0.0, 0.5, 1.0, DSMVC_GB_REPEAT, 0};
    const dsmvc_gb_conversion c{conv.input_offset, conv.input_scale, conv.output_scale, conv.output_offset,
                                conv.output_maximum};
    expect(dsmvc_gb_executor_create(0, &ex) == DSMVC_GB_OK && dsmvc_gb_plan_build(&rh, nullptr, nullptr, &oh) == DSMVC_GB_OK
               && dsmvc_gb_plan_build(&rv, nullptr, nullptr, &ov) == DSMVC_GB_OK
               && dsmvc_gb_inverse_2d_u16(ex, oh, ov, x.data(), 1920, own.data(), 1440, &c) == DSMVC_GB_OK,
           "C ABI call");
    expect(own == got, "bit-identical to the C ABI's own call");
    dsmvc_gb_plan_release(oh);
    dsmvc_gb_plan_release(ov);
    dsmvc_gb_executor_destroy(ex);
    std::printf("dropin gpu ok (max %d code vs the CPU scalar route)\n", worst);
}

} // namespace

int main(int argc, char **argv) {
    const std::string mode = argc > 1 ? argv[1] : "caps";
    try {
        if (mode == "caps") check_caps();
        else if (mode == "gpu") check_gpu();
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
