// Request loop in front of the executor: continuous batching of descale
// requests of mixed sizes, kernels and precisions, admitted by a device
// memory budget.
//
// The reference serves one frame per synchronous call on execution slots
// (src/cuda/cuda_executor.cpp:1462-1503); here requests are queued as they
// arrive and `streams` worker threads each take every admitted request that
// fits the budget (up to `max_batch`) as one batch: host-to-device copies,
// one executor batch of all their planes, device-to-host copies, one wait.
// While a batch runs, requests that arrive are admitted into the next free
// worker's batch as memory frees up, so the batches of different workers
// overlap on the device.  A request's memory (input and output planes plus
// the scratch bound of its planes) comes from one device arena of
// `memory_budget` bytes; a request larger than the budget is refused at
// submission.  Plans are shared pointers, so unprepared plans stay resident
// in the executor's device plan cache across requests.  A request's output
// does not depend on the requests batched with it.
#pragma once

#include "executor.hpp"
#include "planner.hpp"

#include <cstddef>
#include <cstdint>
#include <memory>
#include <string>
#include <vector>

namespace dsmvc_gb {

struct ServePlane {
    std::shared_ptr<const AxisPlan> horizontal, vertical;
    const void *input = nullptr;        // host
    std::ptrdiff_t input_stride = 0;    // samples
    void *output = nullptr;             // host
    std::ptrdiff_t output_stride = 0;   // samples
    dev::Sample sample = dev::Sample::f32;
    IntegerConversion conversion{};
};

struct ServerOptions {
    std::size_t memory_budget = 0;      // device arena bytes; 0 = 8 GiB
    int streams = 4;                    // batches in flight
    int max_batch = 32;                 // requests per batch
};

struct ServerStats {
    std::uint64_t submitted = 0;
    std::uint64_t completed = 0;        // including failed
    std::uint64_t failed = 0;
    std::uint64_t batches = 0;
    double latency_p50_ms = 0.0;        // submission to completion
    double latency_p99_ms = 0.0;
    double latency_mean_ms = 0.0;
    double latency_max_ms = 0.0;
    std::size_t peak_device_bytes = 0;  // arena bytes in use at most
    std::uint64_t source_pixels = 0;    // of completed requests
    double mean_batch_requests = 0.0;
};

class Server {
public:
    Server(Executor &executor, const ServerOptions &options);
    ~Server();   // finishes queued and running requests
    Server(const Server &) = delete;
    Server &operator=(const Server &) = delete;

    // Validates and queues a request; returns its ticket.  The host buffers
    // must stay valid until the request completes.
    std::uint64_t submit(std::vector<ServePlane> planes);
    // Waits for the request; returns 0 or a status code (the C ABI's), the
    // message in `message`.  The ticket is released.
    int wait(std::uint64_t ticket, std::string *message);
    [[nodiscard]] bool done(std::uint64_t ticket) const;
    [[nodiscard]] ServerStats stats() const;
    void reset_stats();

    struct Impl;

private:
    std::unique_ptr<Impl> impl_;
};

} // namespace dsmvc_gb
