// Request loop (server.hpp).
#include "server.hpp"
#include "copy.hpp"

#include "../../include/dsmvc_gb300.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <mutex>
#include <stdexcept>
#include <thread>
#include <unordered_map>

namespace dsmvc_gb {
namespace {

using Clock = std::chrono::steady_clock;

void check(cudaError_t e, const char *what) {
    if (e != cudaSuccess) throw std::runtime_error(std::string("CUDA ") + what + ": " + cudaGetErrorString(e));
}

constexpr std::size_t kAlign = 256;
std::size_t align_up(std::size_t v) { return (v + kAlign - 1) / kAlign * kAlign; }

std::size_t sample_bytes(dev::Sample s) {
    return s == dev::Sample::u8 ? 1 : s == dev::Sample::u16 ? 2 : 4;
}

// First-fit allocator over one device allocation; free blocks coalesce.
class Arena {
public:
    void init(std::size_t bytes) {
        check(cudaMalloc(&base_, bytes), "allocating the request arena");
        size_ = bytes;
        free_[0] = bytes;
    }
    ~Arena() { if (base_) cudaFree(base_); }
    [[nodiscard]] std::size_t largest_free() const {
        std::size_t m = 0;
        for (const auto &[o, n] : free_) m = std::max(m, n);
        return m;
    }
    bool allocate(std::size_t n, std::size_t &offset) {
        n = align_up(std::max<std::size_t>(n, 1));
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second < n) continue;
            offset = it->first;
            const std::size_t rest = it->second - n;
            free_.erase(it);
            if (rest) free_[offset + n] = rest;
            used_ += n;
            peak_ = std::max(peak_, used_);
            return true;
        }
        return false;
    }
    void release(std::size_t offset, std::size_t n) {
        n = align_up(std::max<std::size_t>(n, 1));
        used_ -= n;
        auto it = free_.emplace(offset, n).first;
        if (auto next = std::next(it); next != free_.end() && it->first + it->second == next->first) {
            it->second += next->second;
            free_.erase(next);
        }
        if (it != free_.begin()) {
            auto prev = std::prev(it);
            if (prev->first + prev->second == it->first) {
                prev->second += it->second;
                free_.erase(it);
            }
        }
    }
    [[nodiscard]] char *base() const { return static_cast<char *>(base_); }
    [[nodiscard]] std::size_t size() const { return size_; }
    [[nodiscard]] std::size_t peak() const { return peak_; }
    void reset_peak() { peak_ = used_; }

private:
    void *base_ = nullptr;
    std::size_t size_ = 0, used_ = 0, peak_ = 0;
    std::map<std::size_t, std::size_t> free_;
};

int status_of(const std::exception &e) {
    if (dynamic_cast<const std::invalid_argument *>(&e)) return DSMVC_GB_INVALID_ARGUMENT;
    if (dynamic_cast<const std::length_error *>(&e) || dynamic_cast<const std::out_of_range *>(&e))
        return DSMVC_GB_LENGTH_ERROR;
    if (dynamic_cast<const std::bad_alloc *>(&e)) return DSMVC_GB_OUT_OF_MEMORY;
    const std::string m = e.what();
    if (m.rfind("CUDA", 0) == 0)
        return m.find("out of memory") != std::string::npos ? DSMVC_GB_OUT_OF_MEMORY : DSMVC_GB_CUDA_ERROR;
    return DSMVC_GB_RUNTIME_ERROR;
}

} // namespace

struct Server::Impl {
    struct Request {
        std::uint64_t ticket = 0;
        std::vector<ServePlane> planes;
        std::size_t bytes = 0;          // arena bytes: planes + scratch bound
        bool f64 = false;
        Clock::time_point arrival;
        bool done = false;
        int status = 0;
        std::string message;
    };

    Executor *executor = nullptr;
    ServerOptions options;
    Arena arena;
    mutable std::mutex mutex;
    std::condition_variable work;       // queue or memory changed
    std::condition_variable finished;   // a request completed
    std::deque<std::shared_ptr<Request>> queue;
    std::unordered_map<std::uint64_t, std::shared_ptr<Request>> tickets;
    std::uint64_t next_ticket = 1;
    bool stopping = false;
    std::vector<std::thread> workers;
    std::vector<cudaStream_t> streams;
    // Statistics.
    std::vector<double> latencies;
    ServerStats counters;
    std::uint64_t batch_requests = 0;

    static std::size_t request_bytes(const std::vector<ServePlane> &planes, bool &f64) {
        std::size_t bytes = 0;
        std::vector<PlaneTask> probe;
        f64 = false;
        for (const auto &p : planes) {
            const std::size_t es = sample_bytes(p.sample);
            bytes += align_up(static_cast<std::size_t>(p.horizontal->source_size) * p.vertical->source_size * es);
            bytes += align_up(static_cast<std::size_t>(p.horizontal->destination_size)
                              * p.vertical->destination_size * es);
            PlaneTask t;
            t.horizontal = p.horizontal.get();
            t.vertical = p.vertical.get();
            probe.push_back(t);
            f64 = f64 || p.horizontal->requires_float64() || p.vertical->requires_float64();
        }
        return bytes + Executor::batch_scratch_bound(probe);
    }

    // Uploads the batch's planes, runs them as one executor batch and
    // downloads the results; a Float64 status error is traced to its
    // requests by running the Float64 requests again one at a time.
    void run(std::vector<std::shared_ptr<Request>> &batch, std::size_t offset, std::size_t bytes,
             cudaStream_t s) {
        struct Placed {
            Request *req;
            std::vector<PlaneTask> tasks;
            std::vector<void *> out;
        };
        std::vector<Placed> placed;
        for (auto &r : batch) placed.push_back(Placed{r.get(), {}, {}});
        auto download = [&](const Placed &pl) {
            for (std::size_t i = 0; i < pl.tasks.size(); ++i) {
                const auto &pn = pl.req->planes[i];
                const std::size_t es = sample_bytes(pn.sample);
                const auto &h = *pn.horizontal, &v = *pn.vertical;
                check(copy_plane(pn.output, pn.output_stride * es, pl.out[i], h.destination_size * es,
                                        h.destination_size * es, v.destination_size, cudaMemcpyDeviceToHost, s),
                      "downloading a request plane");
            }
        };
        try {
            char *p = arena.base() + offset;
            char *const end = p + bytes;
            std::vector<PlaneTask> tasks;
            for (auto &pl : placed) {
                for (const auto &pn : pl.req->planes) {
                    const std::size_t es = sample_bytes(pn.sample);
                    const auto &h = *pn.horizontal, &v = *pn.vertical;
                    char *din = p;
                    p += align_up(static_cast<std::size_t>(h.source_size) * v.source_size * es);
                    char *dout = p;
                    p += align_up(static_cast<std::size_t>(h.destination_size) * v.destination_size * es);
                    check(copy_plane(din, h.source_size * es, pn.input, pn.input_stride * es,
                                            h.source_size * es, v.source_size, cudaMemcpyHostToDevice, s),
                          "uploading a request plane");
                    PlaneTask t;
                    t.horizontal = &h;
                    t.vertical = &v;
                    t.horizontal_keep = pn.horizontal;
                    t.vertical_keep = pn.vertical;
                    t.input = din;
                    t.input_stride = h.source_size;
                    t.output = dout;
                    t.output_stride = h.destination_size;
                    t.sample = pn.sample;
                    t.conversion = pn.conversion;
                    pl.tasks.push_back(t);
                    pl.out.push_back(dout);
                    tasks.push_back(t);
                }
            }
            char *scratch = p;
            const auto scratch_bytes = static_cast<std::size_t>(end - p);
            executor->run_batch(tasks, s, false, scratch, scratch_bytes);
            for (const auto &pl : placed) download(pl);
            try {
                executor->check_status(s);
            } catch (const std::runtime_error &e) {
                if (std::string(e.what()).rfind("Float64", 0) != 0) throw;
                for (auto &pl : placed) {
                    if (!pl.req->f64) continue;
                    try {
                        executor->run_batch(pl.tasks, s, true, scratch, scratch_bytes);
                        download(pl);
                        check(cudaStreamSynchronize(s), "synchronizing");
                    } catch (const std::exception &e2) {
                        pl.req->status = status_of(e2);
                        pl.req->message = e2.what();
                    }
                }
            }
        } catch (const std::exception &e) {
            cudaStreamSynchronize(s);
            for (auto &pl : placed) {
                if (pl.req->status) continue;
                pl.req->status = status_of(e);
                pl.req->message = e.what();
            }
        }
    }

    void worker(int index) {
        cudaSetDevice(executor->device());
        cudaStream_t s = streams[static_cast<std::size_t>(index)];
        for (;;) {
            std::vector<std::shared_ptr<Request>> batch;
            std::size_t offset = 0, bytes = 0;
            bool more = false;
            {
                std::unique_lock lock(mutex);
                for (;;) {
                    if (queue.empty()) {
                        if (stopping) return;
                        work.wait(lock);
                        continue;
                    }
                    // Admit from the front while the batch fits the arena.
                    const std::size_t room = arena.largest_free();
                    std::size_t total = 0;
                    for (const auto &r : queue) {
                        if (static_cast<int>(batch.size()) >= options.max_batch) break;
                        if (total + r->bytes > room) break;
                        total += r->bytes;
                        batch.push_back(r);
                    }
                    if (!batch.empty() && arena.allocate(total, offset)) {
                        bytes = total;
                        queue.erase(queue.begin(), queue.begin() + static_cast<std::ptrdiff_t>(batch.size()));
                        more = !queue.empty();
                        break;
                    }
                    batch.clear();
                    work.wait(lock);   // memory frees up when a batch completes
                }
            }
            if (more) work.notify_one();
            run(batch, offset, bytes, s);
            const auto now = Clock::now();
            {
                std::scoped_lock lock(mutex);
                arena.release(offset, bytes);
                counters.batches += 1;
                batch_requests += batch.size();
                for (auto &r : batch) {
                    r->done = true;
                    counters.completed += 1;
                    if (r->status) counters.failed += 1;
                    latencies.push_back(std::chrono::duration<double, std::milli>(now - r->arrival).count());
                    for (const auto &pn : r->planes)
                        counters.source_pixels += static_cast<std::uint64_t>(pn.horizontal->source_size)
                            * static_cast<std::uint64_t>(pn.vertical->source_size);
                }
            }
            work.notify_all();
            finished.notify_all();
        }
    }
};

Server::Server(Executor &executor, const ServerOptions &options) : impl_(std::make_unique<Impl>()) {
    auto &m = *impl_;
    m.executor = &executor;
    m.options = options;
    if (m.options.memory_budget == 0) m.options.memory_budget = 8ULL << 30;
    if (m.options.streams < 1 || m.options.streams > 16 || m.options.max_batch < 1)
        throw std::invalid_argument("server streams must be 1..16 and max_batch positive");
    int previous = -1;
    cudaGetDevice(&previous);
    check(cudaSetDevice(executor.device()), "selecting device");
    m.arena.init(m.options.memory_budget);
    for (int i = 0; i < m.options.streams; ++i) {
        cudaStream_t s = nullptr;
        check(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "creating stream");
        m.streams.push_back(s);
    }
    if (previous >= 0) cudaSetDevice(previous);
    for (int i = 0; i < m.options.streams; ++i) m.workers.emplace_back([this, i] { impl_->worker(i); });
}

Server::~Server() {
    {
        std::scoped_lock lock(impl_->mutex);
        impl_->stopping = true;
    }
    impl_->work.notify_all();
    for (auto &t : impl_->workers) t.join();
    for (auto s : impl_->streams) {
        try {
            impl_->executor->release_stream(s);
        } catch (...) {
        }
        cudaStreamDestroy(s);
    }
}

std::uint64_t Server::submit(std::vector<ServePlane> planes) {
    if (planes.empty()) throw std::invalid_argument("a request needs at least one plane");
    for (const auto &p : planes) {
        if (!p.horizontal || !p.vertical || !p.horizontal->valid() || !p.vertical->valid() || !p.input
            || !p.output || p.input_stride < p.horizontal->source_size
            || p.output_stride < p.horizontal->destination_size || p.sample == dev::Sample::f64)
            throw std::invalid_argument("invalid request plane");
    }
    auto r = std::make_shared<Impl::Request>();
    r->bytes = Impl::request_bytes(planes, r->f64);
    if (align_up(r->bytes) > impl_->arena.size())
        throw std::length_error("request exceeds the server's memory budget");
    r->planes = std::move(planes);
    r->arrival = Clock::now();
    {
        std::scoped_lock lock(impl_->mutex);
        if (impl_->stopping) throw std::runtime_error("server is stopping");
        r->ticket = impl_->next_ticket++;
        impl_->tickets[r->ticket] = r;
        impl_->queue.push_back(r);
        impl_->counters.submitted += 1;
    }
    impl_->work.notify_one();
    return r->ticket;
}

int Server::wait(std::uint64_t ticket, std::string *message) {
    std::unique_lock lock(impl_->mutex);
    auto it = impl_->tickets.find(ticket);
    if (it == impl_->tickets.end()) throw std::invalid_argument("unknown ticket");
    auto r = it->second;
    impl_->finished.wait(lock, [&] { return r->done; });
    impl_->tickets.erase(ticket);
    if (message) *message = r->message;
    return r->status;
}

bool Server::done(std::uint64_t ticket) const {
    std::scoped_lock lock(impl_->mutex);
    auto it = impl_->tickets.find(ticket);
    if (it == impl_->tickets.end()) throw std::invalid_argument("unknown ticket");
    return it->second->done;
}

ServerStats Server::stats() const {
    std::scoped_lock lock(impl_->mutex);
    ServerStats s = impl_->counters;
    s.peak_device_bytes = impl_->arena.peak();
    auto l = impl_->latencies;
    if (!l.empty()) {
        std::sort(l.begin(), l.end());
        auto at = [&](double q) {
            const auto i = static_cast<std::size_t>(q * static_cast<double>(l.size() - 1) + 0.5);
            return l[std::min(i, l.size() - 1)];
        };
        s.latency_p50_ms = at(0.50);
        s.latency_p99_ms = at(0.99);
        double sum = 0.0;
        for (double v : l) sum += v;
        s.latency_mean_ms = sum / static_cast<double>(l.size());
        s.latency_max_ms = l.back();
    }
    if (s.batches) s.mean_batch_requests = static_cast<double>(impl_->batch_requests) / static_cast<double>(s.batches);
    return s;
}

void Server::reset_stats() {
    std::scoped_lock lock(impl_->mutex);
    impl_->latencies.clear();
    const auto submitted = impl_->counters.submitted;
    impl_->counters = ServerStats{};
    impl_->counters.submitted = submitted;
    impl_->batch_requests = 0;
    impl_->arena.reset_peak();
}

} // namespace dsmvc_gb
