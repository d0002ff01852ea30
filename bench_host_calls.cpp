// Per-plane synchronous host calls through the C ABI from many threads, as a
// frame server's filter threads make them (the reference plugin calls one
// Executor::inverse_2d_u16 per plane of each requested frame,
// src/vs_plugin.cpp:1425-1758).  bench.py compiles this file against
// libdsmvc_gb300.so and reports its figure beside the pipelined multi-plane
// call: the same step without Python between the threads and the library.
//
//   bench_host_calls THREADS STEPS FRAMES LUMA_H LUMA_V CHROMA_H CHROMA_V LUMA_CONV CHROMA_CONV
//
// Each *_H / *_V argument is one axis request, 11 comma-separated fields in
// the order of dsmvc_gb_axis_request; each *_CONV one conversion, 5 fields in
// the order of dsmvc_gb_conversion.  A frame is one luma plane and two chroma
// planes; the step's input and output planes lie back to back in one host
// allocation per direction (a frame pool), page-locked through
// dsmvc_gb_host_register.  Prints one JSON line.
#include "dsmvc_gb300.h"

#include <atomic>
#include <barrier>
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

namespace {

[[noreturn]] void fail(const std::string &what) {
    std::printf("{\"error\": \"%s: %s\"}\n", what.c_str(), dsmvc_gb_last_error());
    std::exit(1);
}

std::vector<double> fields(const char *text, std::size_t count) {
    std::vector<double> out;
    const char *p = text;
    while (*p) {
        char *end = nullptr;
        out.push_back(std::strtod(p, &end));
        if (end == p) break;
        p = *end == ',' ? end + 1 : end;
    }
    if (out.size() != count) fail(std::string("expected ") + std::to_string(count) + " fields in " + text);
    return out;
}

dsmvc_gb_axis_request request(const char *text) {
    const auto f = fields(text, 11);
    dsmvc_gb_axis_request r{};
    r.source_size = static_cast<int32_t>(f[0]);
    r.destination_size = static_cast<int32_t>(f[1]);
    r.active_length = f[2];
    r.shift = f[3];
    r.kernel = static_cast<int32_t>(f[4]);
    r.taps = static_cast<int32_t>(f[5]);
    r.b = f[6];
    r.c = f[7];
    r.blur = f[8];
    r.border = static_cast<int32_t>(f[9]);
    r.f64_mode = static_cast<int32_t>(f[10]);
    return r;
}

dsmvc_gb_conversion conversion(const char *text) {
    const auto f = fields(text, 5);
    return {static_cast<float>(f[0]), static_cast<float>(f[1]), static_cast<float>(f[2]),
            static_cast<float>(f[3]), static_cast<uint32_t>(f[4])};
}

struct Plane {
    const dsmvc_gb_plan *h, *v;
    const dsmvc_gb_conversion *conv;
    const uint16_t *in;
    uint16_t *out;
    int64_t in_stride, out_stride;
};

} // namespace

int main(int argc, char **argv) {
    if (argc != 10) {
        std::printf("{\"error\": \"usage: bench_host_calls THREADS STEPS FRAMES LUMA_H LUMA_V CHROMA_H "
                    "CHROMA_V LUMA_CONV CHROMA_CONV\"}\n");
        return 2;
    }
    const int threads = std::atoi(argv[1]), steps = std::atoi(argv[2]), frames = std::atoi(argv[3]);
    if (threads < 1 || steps < 1 || frames < 1) fail("invalid counts");
    dsmvc_gb_axis_request req[4] = {request(argv[4]), request(argv[5]), request(argv[6]), request(argv[7])};
    const dsmvc_gb_conversion conv[2] = {conversion(argv[8]), conversion(argv[9])};

    dsmvc_gb_executor *ex = nullptr;
    if (dsmvc_gb_executor_create(0, &ex) != DSMVC_GB_OK) fail("creating the executor");
    dsmvc_gb_plan *plan[4] = {};
    for (int i = 0; i < 4; ++i) {
        if (dsmvc_gb_plan_build(&req[i], nullptr, nullptr, &plan[i]) != DSMVC_GB_OK) fail("building a plan");
        if (dsmvc_gb_prepare(ex, plan[i]) != DSMVC_GB_OK) fail("preparing a plan");
    }
    if (dsmvc_gb_seal(ex) != DSMVC_GB_OK) fail("sealing");

    // Planes of the step: luma, then the two chroma planes, frame after frame.
    std::size_t in_samples = 0, out_samples = 0;
    for (int f = 0; f < frames; ++f)
        for (int k = 0; k < 3; ++k) {
            const int a = k == 0 ? 0 : 2;
            in_samples += static_cast<std::size_t>(req[a].source_size) * req[a + 1].source_size;
            out_samples += static_cast<std::size_t>(req[a].destination_size) * req[a + 1].destination_size;
        }
    std::vector<uint16_t> in(in_samples), out(out_samples);
    int32_t in_locked = -1, out_locked = -1;
    if (dsmvc_gb_host_register(in.data(), static_cast<int64_t>(in.size() * 2), &in_locked) != DSMVC_GB_OK ||
        dsmvc_gb_host_register(out.data(), static_cast<int64_t>(out.size() * 2), &out_locked) != DSMVC_GB_OK)
        fail("page-locking the frames");
    std::uint32_t state = 12345;
    for (auto &x : in) {
        state = state * 1664525U + 1013904223U;
        x = static_cast<uint16_t>(4096 + (state >> 8) % 56064);
    }
    std::vector<Plane> planes;
    std::size_t at_in = 0, at_out = 0;
    for (int f = 0; f < frames; ++f)
        for (int k = 0; k < 3; ++k) {
            const int a = k == 0 ? 0 : 2;
            Plane p{plan[a], plan[a + 1], &conv[k == 0 ? 0 : 1], in.data() + at_in, out.data() + at_out,
                    req[a].source_size, req[a].destination_size};
            planes.push_back(p);
            at_in += static_cast<std::size_t>(req[a].source_size) * req[a + 1].source_size;
            at_out += static_cast<std::size_t>(req[a].destination_size) * req[a + 1].destination_size;
        }

    // Thread t takes planes t, t + threads, ...; every thread meets the
    // others at the end of a step.
    std::atomic<bool> error{false};
    std::barrier sync(threads + 1);
    std::vector<std::thread> pool;
    const int total = steps + 2;   // two warm-up steps
    for (int t = 0; t < threads; ++t)
        pool.emplace_back([&, t] {
            for (int s = 0; s < total; ++s) {
                sync.arrive_and_wait();
                for (std::size_t i = t; i < planes.size(); i += threads) {
                    const Plane &p = planes[i];
                    if (dsmvc_gb_inverse_2d_u16(ex, p.h, p.v, p.in, p.in_stride, p.out, p.out_stride, p.conv) !=
                        DSMVC_GB_OK)
                        error = true;
                }
                sync.arrive_and_wait();
            }
        });
    std::chrono::steady_clock::time_point t0;
    for (int s = 0; s < total; ++s) {
        if (s == 2) t0 = std::chrono::steady_clock::now();
        sync.arrive_and_wait();
        sync.arrive_and_wait();
    }
    const double seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    for (auto &th : pool) th.join();
    if (error) fail("a plane call");
    double pixels = 0;
    for (int f = 0; f < frames; ++f)
        pixels += static_cast<double>(req[0].source_size) * req[1].source_size
            + 2.0 * req[2].source_size * req[3].source_size;
    std::printf("{\"threads\": %d, \"steps\": %d, \"planes_per_step\": %zu, \"ms_per_step\": %.4f, "
                "\"mpix_s\": %.1f, \"frames_page_locked\": %s}\n",
                threads, steps, planes.size(), seconds / steps * 1e3, pixels * steps / seconds / 1e6,
                in_locked >= 0 && out_locked >= 0 ? "true" : "false");
    if (in_locked == 0) dsmvc_gb_host_unregister(in.data());
    if (out_locked == 0) dsmvc_gb_host_unregister(out.data());
    for (auto *p : plan) dsmvc_gb_plan_release(p);
    dsmvc_gb_executor_destroy(ex);
    return 0;
}
