// Batched candidate sweep (sweep.hpp).
#include "sweep.hpp"

#include "score.cuh"
#include "stream.cuh"

#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <chrono>
#include <climits>
#include <cstdint>
#include <iterator>
#include <cstring>
#include <map>
#include <stdexcept>
#include <string>

namespace dsmvc_gb {
namespace {

void check(cudaError_t e, const char *what) {
    if (e != cudaSuccess) throw std::runtime_error(std::string("CUDA ") + what + ": " + cudaGetErrorString(e));
}
void check(int e, const char *what) { check(static_cast<cudaError_t>(e), what); }

constexpr std::size_t kAlign = 256;
std::size_t align_up(std::size_t v) { return (v + kAlign - 1) / kAlign * kAlign; }

struct Buffer {
    void *ptr = nullptr;
    std::size_t bytes = 0;
    Buffer() = default;
    Buffer(const Buffer &) = delete;
    Buffer &operator=(const Buffer &) = delete;
    ~Buffer() { if (ptr) cudaFree(ptr); }
    void allocate(std::size_t n) {
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        bytes = 0;
        check(cudaMalloc(&ptr, std::max<std::size_t>(n, kAlign)), "allocating sweep buffer");
        bytes = n;
    }
    [[nodiscard]] char *data() const { return static_cast<char *>(ptr); }
};

// A (source x destination) as a CSR by source sample, from the plan's CSR
// of A^T: entries keep ascending destination order.
struct HostForward {
    std::vector<std::uint32_t> offsets;
    std::vector<std::int32_t> indices;
    std::vector<float> weights;
};

HostForward forward_csr(const AxisPlan &p) {
    HostForward f;
    const auto n = static_cast<std::size_t>(p.source_size);
    f.offsets.assign(n + 1, 0);
    for (std::size_t j = 0; j < static_cast<std::size_t>(p.destination_size); ++j)
        for (std::uint32_t e = p.transpose_offsets[j]; e < p.transpose_offsets[j + 1]; ++e)
            ++f.offsets[static_cast<std::size_t>(p.transpose_indices[e]) + 1];
    for (std::size_t s = 0; s < n; ++s) f.offsets[s + 1] += f.offsets[s];
    f.indices.resize(f.offsets[n]);
    f.weights.resize(f.offsets[n]);
    std::vector<std::uint32_t> fill(f.offsets.begin(), f.offsets.end() - 1);
    for (std::size_t j = 0; j < static_cast<std::size_t>(p.destination_size); ++j) {
        for (std::uint32_t e = p.transpose_offsets[j]; e < p.transpose_offsets[j + 1]; ++e) {
            const auto s = static_cast<std::size_t>(p.transpose_indices[e]);
            f.indices[fill[s]] = static_cast<std::int32_t>(j);
            f.weights[fill[s]] = p.transpose_weights[e];
            ++fill[s];
        }
    }
    return f;
}

// Dense operator rows of the fused scoring (dev::ScoreEpilogue): 12 floats
// a row.  `ok` is false where an operator does not fit: an empty row or a
// window wider than `max_taps`.  (Windows need not move monotonically: a
// sample that falls on a descaled sample has one entry, narrower than its
// neighbours'.)
struct DenseRows {
    bool ok = false;
    int taps = 0;               // 4 or 8
    int widest = 0;             // largest last - first index of a row
    std::vector<float> rows;    // 12 floats a row
    std::vector<int> first, last;
};

DenseRows dense_rows(const HostForward &f, int max_taps) {
    DenseRows d;
    const int n = static_cast<int>(f.offsets.size()) - 1;
    d.first.resize(static_cast<std::size_t>(n));
    d.last.resize(static_cast<std::size_t>(n));
    for (int r = 0; r < n; ++r) {
        const std::uint32_t e0 = f.offsets[static_cast<std::size_t>(r)], e1 = f.offsets[static_cast<std::size_t>(r) + 1];
        if (e0 == e1) return d;
        const int a = f.indices[e0], b = f.indices[e1 - 1];
        d.first[static_cast<std::size_t>(r)] = a;
        d.last[static_cast<std::size_t>(r)] = b;
        d.widest = std::max(d.widest, b - a);
    }
    if (d.widest + 1 > max_taps) return d;
    d.taps = d.widest + 1 <= 4 ? 4 : 8;
    d.ok = true;
    return d;
}

// Fills row r's window from `start` (weights at index - start).
void put_dense(std::vector<float> &out, const HostForward &f, int r, int start) {
    float *row = out.data() + static_cast<std::size_t>(r) * 12;
    std::int32_t bits = start;
    std::memcpy(row, &bits, 4);
    for (std::uint32_t e = f.offsets[static_cast<std::size_t>(r)]; e < f.offsets[static_cast<std::size_t>(r) + 1]; ++e)
        row[4 + (f.indices[e] - start)] = f.weights[e];
}

} // namespace

constexpr int kSegments[] = {16, 32, 64, 128};        // multiples of kScoreRowBlock
constexpr int kMaxSpanRows = 192;   // staged row-pass rows per scoring block (192 KiB + 16 KiB)

struct Sweep::Impl {
    Executor *executor = nullptr;
    std::vector<std::pair<const AxisPlan *, const AxisPlan *>> candidates;
    std::vector<Sweep::Candidate> owners;
    const float *frame = nullptr;
    std::ptrdiff_t frame_stride = 0;
    int width = 0, height = 0;
    SweepOptions options;
    cudaStream_t stream = nullptr;          // tuning and capture

    struct Wave {
        int first = 0, count = 0;
        std::vector<PlaneTask> tasks;
        std::unique_ptr<PreparedBatch> batch;
        int column_blocks = 0;
        std::array<int, 4> max_span{};   // per entry of kSegments (unfused candidates)
        int fused_first = 0, fused = 0;       // its fused candidates' epilogues
        int unfused_first = 0, unfused = 0;   // its unfused candidates' score jobs
    };
    std::vector<Wave> waves;
    std::vector<std::size_t> y_offset, partial_offset;   // within a wave's buffers
    Buffer forward_mem, y_mem, partial_mem, scratch_mem, job_mem, plain_job_mem, score_mem;
    // Fused scoring (dev::ScoreEpilogue): per candidate its epilogue index
    // (-1: descaled to HBM and scored by score_tiles_kernel) and tile count;
    // the epilogues of fused candidates in candidate order, the unfused
    // candidates' score jobs likewise.
    std::vector<int> epilogue_of, tiles_of, unfused_of;
    int fused_count = 0, unfused_count = 0;
    Buffer epilogue_mem;
    const dev::ScoreEpilogue *epilogues = nullptr;
    // Per vertical plan and segment length: the most descaled rows one
    // segment of source rows touches.
    std::map<const AxisPlan *, std::array<int, 4>> spans;
    std::size_t scratch_capacity = 0;
    std::map<const AxisPlan *, dev::ForwardCsr> forward;
    std::map<const AxisPlan *, HostForward> host_forward;   // while building
    int segment_rows = 32;
    int best_segment = 32;
    int vectors_per_warp = 0;   // 0: the executor's default; 32 / 64 once tuned
    BatchTuning tuning;
    double tune_ms = 0.0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t graph_exec = nullptr;

    ~Impl() {
        if (stream) cudaStreamSynchronize(stream);
        if (graph_exec) cudaGraphExecDestroy(graph_exec);
        if (graph) cudaGraphDestroy(graph);
        if (stream) cudaStreamDestroy(stream);
    }

    void upload_forward() {
        std::size_t bytes = 0;
        for (const auto &[h, v] : candidates) {
            for (const AxisPlan *p : {h, v}) {
                if (host_forward.count(p)) continue;
                auto f = forward_csr(*p);
                bytes += align_up(f.offsets.size() * 4) + align_up(f.indices.size() * 4)
                    + align_up(f.weights.size() * 4);
                host_forward.emplace(p, std::move(f));
            }
        }
        std::vector<char> blob(std::max<std::size_t>(bytes, kAlign), 0);
        forward_mem.allocate(blob.size());
        std::size_t at = 0;
        for (auto &[p, f] : host_forward) {
            dev::ForwardCsr c{};
            auto put = [&](const void *src, std::size_t n) {
                std::memcpy(blob.data() + at, src, n);
                const char *d = forward_mem.data() + at;
                at += align_up(n);
                return d;
            };
            c.offsets = reinterpret_cast<const std::uint32_t *>(put(f.offsets.data(), f.offsets.size() * 4));
            c.indices = reinterpret_cast<const std::int32_t *>(put(f.indices.data(), f.indices.size() * 4));
            c.weights = reinterpret_cast<const float *>(put(f.weights.data(), f.weights.size() * 4));
            forward[p] = c;
            std::array<int, 4> sp{};
            for (std::size_t k = 0; k < sp.size(); ++k) {
                const int seg = kSegments[k];
                const int rows = static_cast<int>(f.offsets.size()) - 1;
                for (int r0 = 0; r0 < rows; r0 += seg) {
                    int lo = INT32_MAX, hi = -1;
                    for (int r = r0; r < std::min(rows, r0 + seg); ++r) {
                        if (f.offsets[r] < f.offsets[r + 1]) {
                            lo = std::min(lo, f.indices[f.offsets[r]]);
                            hi = std::max(hi, f.indices[f.offsets[r + 1] - 1]);
                        }
                    }
                    if (hi >= lo) sp[k] = std::max(sp[k], hi - lo + 1);
                }
            }
            spans[p] = sp;
        }
        check(cudaMemcpy(forward_mem.data(), blob.data(), blob.size(), cudaMemcpyHostToDevice),
              "uploading forward operators");
    }

    // Decides per candidate whether its scoring fuses into its columns pass
    // (the executor runs that pass with the fused kernel and both operators
    // fit the epilogue's windows) and uploads the fused candidates' operator
    // tables, tile bounds, partial sums and epilogues.
    void build_epilogues() {
        const std::size_t n = candidates.size();
        epilogue_of.assign(n, -1);
        tiles_of.assign(n, 0);
        unfused_of.assign(n, -1);
        struct VTable {
            DenseRows d;
            std::vector<std::int32_t> emit;
        };
        struct HTable {
            DenseRows d;
            int tiles = 0;
            std::vector<std::int32_t> sources, origins;
        };
        std::map<const AxisPlan *, VTable> vtab;
        std::map<const AxisPlan *, HTable> htab;
        std::map<const AxisPlan *, int> windows;
        auto vertical_table = [&](const AxisPlan *v) -> const VTable & {
            auto it = vtab.find(v);
            if (it != vtab.end()) return it->second;
            VTable t;
            const HostForward &f = host_forward.at(v);
            t.d = dense_rows(f, kScoreMaxVerticalTaps);
            if (t.d.ok) {
                const int rows = static_cast<int>(f.offsets.size()) - 1;
                const int chunks = (v->destination_size + kStreamChunk - 1) / kStreamChunk;
                t.d.rows.assign(static_cast<std::size_t>(rows) * 12, 0.0f);
                t.emit.assign(static_cast<std::size_t>(chunks), 0);
                // A row is re-upscaled after the first chunk that holds its
                // last entry and every earlier row's; its window then lies in
                // that chunk and the ring rows before it.
                int q = 0;
                for (int r = 0; r < rows && t.d.ok; ++r) {
                    q = std::max(q, t.d.last[static_cast<std::size_t>(r)] / kStreamChunk);
                    const int start = std::min(t.d.first[static_cast<std::size_t>(r)],
                                               kStreamChunk * (q + 1) - t.d.taps);
                    // The window's ring slots: [start - (32 q - halo), + taps)
                    // within the kScoreRingRows the kernel keeps.
                    const int slot = start - (kStreamChunk * q - (kScoreRingRows - kStreamChunk));
                    if (q >= chunks || slot < 0 || slot + t.d.taps > kScoreRingRows) t.d.ok = false;
                    else put_dense(t.d.rows, f, r, start);
                    t.emit[static_cast<std::size_t>(q < chunks ? q : 0)] = r + 1;
                }
                for (int c = 1; c < chunks; ++c)
                    t.emit[static_cast<std::size_t>(c)] = std::max(t.emit[static_cast<std::size_t>(c)],
                                                                   t.emit[static_cast<std::size_t>(c) - 1]);
                if (chunks < 1 || t.emit.back() != rows) t.d.ok = false;
            }
            return vtab.emplace(v, std::move(t)).first->second;
        };
        auto horizontal_table = [&](const AxisPlan *h) -> const HTable & {
            auto it = htab.find(h);
            if (it != htab.end()) return it->second;
            HTable t;
            const HostForward &f = host_forward.at(h);
            t.d = dense_rows(f, kScoreMaxHorizontalTaps);
            if (t.d.ok) {
                const int cols = static_cast<int>(f.offsets.size()) - 1;
                t.d.rows.assign(static_cast<std::size_t>(cols) * 12, 0.0f);
                for (int s = 0; s < cols; ++s) put_dense(t.d.rows, f, s, t.d.first[static_cast<std::size_t>(s)]);
                // Tiles: runs of consecutive source columns as long as their
                // windows lie within kScoreCtaThreads descaled columns from
                // the run's lowest window start (the tile's origin) and their
                // padded windows within the row buffer's 8 zero columns after.
                for (int s = 0; s < cols;) {
                    int lo = t.d.first[static_cast<std::size_t>(s)], hi = -1, pad = 0, e = s;
                    for (; e < cols; ++e) {
                        const int nlo = std::min(lo, t.d.first[static_cast<std::size_t>(e)]);
                        const int nhi = std::max(hi, t.d.last[static_cast<std::size_t>(e)]);
                        const int npad = std::max(pad, t.d.first[static_cast<std::size_t>(e)] + t.d.taps);
                        if (e > s && (nhi - nlo >= kScoreCtaThreads || npad - nlo > kScoreCtaThreads + 8)) break;
                        lo = nlo;
                        hi = nhi;
                        pad = npad;
                    }
                    t.sources.push_back(s);
                    t.origins.push_back(lo);
                    s = e;
                }
                t.sources.push_back(cols);
                t.tiles = static_cast<int>(t.origins.size());
            }
            return htab.emplace(h, std::move(t)).first->second;
        };
        for (std::size_t i = 0; i < n; ++i) {
            const auto &[h, v] = candidates[i];
            bool ok = options.fused_scoring;
            if (ok) {
                auto w = windows.find(v);
                if (w == windows.end()) w = windows.emplace(v, executor->fused_scoring_window(*v, owners[i].second)).first;
                ok = w->second >= 0;
            }
            ok = ok && vertical_table(v).d.ok && horizontal_table(h).d.ok;
            if (ok) {
                epilogue_of[i] = fused_count++;
                tiles_of[i] = htab.at(h).tiles;
            } else {
                unfused_of[i] = unfused_count++;
            }
        }
        if (!fused_count) return;
        // One allocation: the tables, then each fused candidate's partials,
        // then the epilogues.
        std::size_t bytes = 0;
        std::map<const AxisPlan *, std::size_t> at_v, at_h;
        for (std::size_t i = 0; i < n; ++i) {
            if (epilogue_of[i] < 0) continue;
            const auto &[h, v] = candidates[i];
            if (!at_v.count(v)) {
                at_v[v] = bytes;
                const auto &t = vtab.at(v);
                bytes += align_up(t.d.rows.size() * 4) + align_up(t.emit.size() * 4);
            }
            if (!at_h.count(h)) {
                at_h[h] = bytes;
                const auto &t = htab.at(h);
                bytes += align_up(t.d.rows.size() * 4) + align_up(t.sources.size() * 4)
                    + align_up(t.origins.size() * 4);
            }
        }
        std::vector<std::size_t> at_partials(n, 0);
        for (std::size_t i = 0; i < n; ++i) {
            if (epilogue_of[i] < 0) continue;
            at_partials[i] = bytes;
            bytes += align_up(static_cast<std::size_t>(tiles_of[i]) * sizeof(double));
        }
        const std::size_t at_epilogues = bytes;
        bytes += static_cast<std::size_t>(fused_count) * sizeof(dev::ScoreEpilogue);
        std::vector<char> blob(bytes, 0);
        epilogue_mem.allocate(bytes);
        char *base = epilogue_mem.data();
        auto put = [&](std::size_t at, const void *src, std::size_t len) {
            if (len) std::memcpy(blob.data() + at, src, len);
        };
        for (const auto &[v, at] : at_v) {
            const auto &t = vtab.at(v);
            put(at, t.d.rows.data(), t.d.rows.size() * 4);
            put(at + align_up(t.d.rows.size() * 4), t.emit.data(), t.emit.size() * 4);
        }
        for (const auto &[h, at] : at_h) {
            const auto &t = htab.at(h);
            put(at, t.d.rows.data(), t.d.rows.size() * 4);
            put(at + align_up(t.d.rows.size() * 4), t.sources.data(), t.sources.size() * 4);
            put(at + align_up(t.d.rows.size() * 4) + align_up(t.sources.size() * 4), t.origins.data(),
                t.origins.size() * 4);
        }
        auto *eps = reinterpret_cast<dev::ScoreEpilogue *>(blob.data() + at_epilogues);
        for (std::size_t i = 0; i < n; ++i) {
            if (epilogue_of[i] < 0) continue;
            const auto &[h, v] = candidates[i];
            const auto &vt = vtab.at(v);
            const auto &ht = htab.at(h);
            dev::ScoreEpilogue e{};
            e.frame = frame;
            e.frame_stride = frame_stride;
            e.width = width;
            e.height = height;
            e.v_rows = reinterpret_cast<const float *>(base + at_v.at(v));
            e.v_emit = reinterpret_cast<const std::int32_t *>(base + at_v.at(v) + align_up(vt.d.rows.size() * 4));
            e.h_cols = reinterpret_cast<const float *>(base + at_h.at(h));
            e.tile_sources = reinterpret_cast<const std::int32_t *>(base + at_h.at(h)
                                                                    + align_up(ht.d.rows.size() * 4));
            e.tile_origins = e.tile_sources + align_up(ht.sources.size() * 4) / 4;
            e.v_taps = vt.d.taps;
            e.h_taps = ht.d.taps;
            e.tiles = ht.tiles;
            e.partials = reinterpret_cast<double *>(base + at_partials[i]);
            e.score = reinterpret_cast<float *>(score_mem.data()) + i;
            eps[epilogue_of[i]] = e;
        }
        check(cudaMemcpy(base, blob.data(), bytes, cudaMemcpyHostToDevice), "uploading fused scoring tables");
        epilogues = reinterpret_cast<const dev::ScoreEpilogue *>(base + at_epilogues);
    }

    [[nodiscard]] int column_tiles() const { return (width + kScoreThreads - 1) / kScoreThreads; }
    [[nodiscard]] int segments(int seg) const { return (height + seg - 1) / seg; }

    // Splits the candidates into waves within the memory budget and lays
    // out each wave's descaled planes (unfused candidates), row-pass scratch
    // and partial sums.
    void plan_waves() {
        const std::size_t budget = options.memory_budget ? options.memory_budget : (32ULL << 30);
        const std::size_t partials = align_up(static_cast<std::size_t>(column_tiles()) * segments(kScoreRowBlock) * 4);
        std::size_t y_bytes = 0, p_bytes = 0, s_bytes = 0;
        std::size_t y_max = 0, p_max = 0, s_max = 0;
        y_offset.assign(candidates.size(), 0);
        partial_offset.assign(candidates.size(), 0);
        Wave cur;
        int fused_seen = 0, unfused_seen = 0;
        auto task_of = [&](std::size_t i) {
            PlaneTask t;
            t.horizontal = candidates[i].first;
            t.vertical = candidates[i].second;
            t.horizontal_keep = owners[i].first;
            t.vertical_keep = owners[i].second;
            t.input = frame;
            t.input_stride = frame_stride;
            t.output_stride = candidates[i].first->destination_size;
            t.sample = dev::Sample::f32;
            if (epilogue_of[i] >= 0) {
                t.score = epilogues + epilogue_of[i];
                t.score_tiles = tiles_of[i];
            }
            return t;
        };
        for (std::size_t i = 0; i < candidates.size(); ++i) {
            const auto &[h, v] = candidates[i];
            const bool fused = epilogue_of[i] >= 0;
            const std::size_t y = fused ? 0 : align_up(static_cast<std::size_t>(h->destination_size) * v->destination_size * 4);
            const std::size_t part = fused ? 0 : partials;
            const std::size_t s = Executor::batch_scratch_bound({task_of(i)});
            if (cur.count > 0 && y_bytes + p_bytes + s_bytes + y + part + s > budget) {
                waves.push_back(std::move(cur));
                cur = Wave{};
                y_bytes = p_bytes = s_bytes = 0;
            }
            if (cur.count == 0) {
                cur.first = static_cast<int>(i);
                cur.fused_first = fused_seen;
                cur.unfused_first = unfused_seen;
            }
            ++cur.count;
            if (fused) {
                ++cur.fused;
                ++fused_seen;
            } else {
                ++cur.unfused;
                ++unfused_seen;
                y_offset[i] = y_bytes;
                partial_offset[i] = p_bytes;
                const auto &sp = spans.at(v);
                for (std::size_t k = 0; k < sp.size(); ++k) cur.max_span[k] = std::max(cur.max_span[k], sp[k]);
            }
            y_bytes += y;
            p_bytes += part;
            s_bytes += s;
            y_max = std::max(y_max, y_bytes);
            p_max = std::max(p_max, p_bytes);
            s_max = std::max(s_max, s_bytes);
        }
        if (cur.count > 0) waves.push_back(std::move(cur));
        y_mem.allocate(y_max);
        partial_mem.allocate(p_max);
        scratch_mem.allocate(s_max);
        scratch_capacity = s_max;
        for (auto &w : waves) {
            for (int k = 0; k < w.count; ++k) {
                const std::size_t i = static_cast<std::size_t>(w.first + k);
                PlaneTask t = task_of(i);
                if (epilogue_of[i] < 0) t.output = y_mem.data() + y_offset[i];
                w.tasks.push_back(t);
            }
        }
    }

    // Score jobs of the unfused candidates (in candidate order) with `seg`
    // source rows per column-pass block; block numbering restarts at each
    // wave (`plain`: at each job).
    std::vector<dev::ScoreJob> score_jobs(int seg, bool plain) {
        std::vector<dev::ScoreJob> jobs(static_cast<std::size_t>(unfused_count));
        for (auto &w : waves) {
            int cols = 0;
            for (int k = 0; k < w.count; ++k) {
                const std::size_t i = static_cast<std::size_t>(w.first + k);
                if (unfused_of[i] < 0) continue;
                const AxisPlan *h = candidates[i].first, *v = candidates[i].second;
                auto &j = jobs[static_cast<std::size_t>(unfused_of[i])];
                j.descaled = reinterpret_cast<const float *>(y_mem.data() + y_offset[i]);
                j.descaled_stride = h->destination_size;
                j.rows = v->destination_size;
                j.cols = h->destination_size;
                j.frame = frame;
                j.frame_stride = frame_stride;
                j.width = width;
                j.height = height;
                j.h = forward.at(h);
                j.v = forward.at(v);
                j.partials = reinterpret_cast<float *>(partial_mem.data() + partial_offset[i]);
                j.score = reinterpret_cast<float *>(score_mem.data()) + i;
                j.segment_rows = seg;
                j.column_tiles = column_tiles();
                j.first_block = plain ? 0 : cols;
                cols += j.column_tiles * segments(seg);
            }
            w.column_blocks = cols;
        }
        return jobs;
    }

    void upload_jobs(Buffer &mem, const std::vector<dev::ScoreJob> &jobs) {
        const std::size_t n = std::max<std::size_t>(jobs.size(), 1) * sizeof(dev::ScoreJob);
        if (mem.bytes < n) mem.allocate(n);
        if (!jobs.empty())
            check(cudaMemcpy(mem.data(), jobs.data(), jobs.size() * sizeof(dev::ScoreJob), cudaMemcpyHostToDevice),
                  "uploading score jobs");
    }

    [[nodiscard]] const dev::ScoreJob *wave_jobs(const Wave &w) const {
        return reinterpret_cast<const dev::ScoreJob *>(job_mem.data()) + w.unfused_first;
    }

    [[nodiscard]] int span_rows(const Wave &w) const {
        for (std::size_t k = 0; k < std::size(kSegments); ++k)
            if (kSegments[k] == segment_rows) return w.max_span[k];
        return 0;
    }

    // A wave's scores are reduced before the next wave reuses its buffers
    // (descaled planes and partial sums).
    void enqueue_scoring(const Wave &w, cudaStream_t s) {
        if (w.unfused) {
            check(launch_score_tiles(wave_jobs(w), w.unfused, w.column_blocks, span_rows(w), s), "launching scoring");
            check(launch_score_finalize(wave_jobs(w), w.unfused, s), "launching score finalize");
        }
        if (w.fused)
            check(launch_fused_score_finalize(epilogues + w.fused_first, w.fused, s), "launching score finalize");
    }

    void enqueue_all(cudaStream_t s) {
        for (auto &w : waves) {
            w.batch->launch(s);
            enqueue_scoring(w, s);
        }
    }

    template <class F> float time_ms(F &&f, int reps) {
        cudaEvent_t a = nullptr, b = nullptr;
        check(cudaEventCreate(&a), "creating event");
        check(cudaEventCreate(&b), "creating event");
        f();   // warm
        check(cudaEventRecord(a, stream), "recording event");
        for (int r = 0; r < reps; ++r) f();
        check(cudaEventRecord(b, stream), "recording event");
        check(cudaEventSynchronize(b), "waiting for event");
        float ms = 0.0F;
        check(cudaEventElapsedTime(&ms, a, b), "reading event");
        cudaEventDestroy(a);
        cudaEventDestroy(b);
        return ms / static_cast<float>(reps);
    }

    // Times the first wave's descale with one and with two right-hand sides
    // a lane (32 or 64 vectors a warp), then every launch group of it at
    // each candidate CTA size, and the scoring column pass at each row
    // segment (unfused candidates); keeps the fastest of each.  Scores do
    // not depend on the choices: every kernel variant gives each output bit
    // for bit, and the fused scoring kernel has one launch shape.
    void autotune() {
        const auto t0 = std::chrono::steady_clock::now();
        Wave &w = waves.front();
        // Two right-hand sides a lane only where some plan admits the paired
        // kernels: otherwise both batches are the same launches.
        auto single = executor->prepare_batch(w.tasks, nullptr, scratch_mem.data(), scratch_capacity, 32);
        auto paired = executor->prepare_batch(w.tasks, nullptr, scratch_mem.data(), scratch_capacity, 64);
        const auto paired_groups = paired->groups();
        vectors_per_warp = 32;
        if (std::any_of(paired_groups.begin(), paired_groups.end(), [](const BatchGroup &g) { return g.kind == 4; })) {
            const float ms32 = time_ms([&] { single->launch(stream); }, 2);
            const float ms64 = time_ms([&] { paired->launch(stream); }, 2);
            check(cudaStreamSynchronize(stream), "synchronizing");
            if (ms64 < ms32) vectors_per_warp = 64;
        }
        std::map<std::array<int, 6>, std::pair<float, int>> best;
        const auto keys = (vectors_per_warp == 64 ? paired : single)->groups();
        single.reset();
        paired.reset();
        // 32-thread CTAs never win on these kernels (one warp per record copy).
        for (const int threads : {64, 128, 256}) {
            BatchTuning all;
            for (const auto &g : keys) {
                const int most = g.kind >= 3 ? 256 : 128;
                if (g.kind != 2 && g.kind <= 6 && threads <= most) all[g.key] = threads;
            }
            if (all.empty()) continue;
            auto batch = executor->prepare_batch(w.tasks, &all, scratch_mem.data(), scratch_capacity,
                                                 vectors_per_warp);
            const auto groups = batch->groups();
            for (std::size_t gi = 0; gi < groups.size(); ++gi) {
                if (!all.count(groups[gi].key)) continue;
                const float ms = time_ms([&] { batch->launch_group(gi, stream); }, 1);
                auto it = best.find(groups[gi].key);
                if (it == best.end() || ms < it->second.first) best[groups[gi].key] = {ms, threads};
            }
            check(cudaStreamSynchronize(stream), "synchronizing");
        }
        tuning.clear();
        for (const auto &[k, v] : best) tuning[k] = v.second;
        float best_ms = 0.0F;
        const int fallback = segment_rows;
        bool any = false;
        for (std::size_t k = 0; w.unfused && k < std::size(kSegments); ++k) {
            if (w.max_span[k] > kMaxSpanRows) continue;
            upload_jobs(job_mem, score_jobs(kSegments[k], false));
            segment_rows = kSegments[k];
            const float ms = time_ms([&] {
                check(launch_score_tiles(wave_jobs(w), w.unfused, w.column_blocks, span_rows(w), stream), "launching");
            }, 1);
            if (!any || ms < best_ms) {
                best_ms = ms;
                any = true;
                best_segment = kSegments[k];
            }
        }
        segment_rows = any ? best_segment : fallback;
        tune_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    }

    void build() {
        check(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "creating stream");
        score_mem.allocate(candidates.size() * sizeof(float));
        upload_forward();
        build_epilogues();
        host_forward.clear();
        plan_waves();
        if (options.autotune) autotune();
        // Every wave's row span at the chosen segment must fit the staging.
        for (const auto &w : waves) {
            while (span_rows(w) > kMaxSpanRows && segment_rows > kSegments[0]) segment_rows /= 2;
            if (span_rows(w) > kMaxSpanRows) throw std::length_error("candidate too far from its source size to score");
        }
        for (auto &w : waves)
            w.batch = executor->prepare_batch(w.tasks, &tuning, scratch_mem.data(), scratch_capacity,
                                              vectors_per_warp);
        upload_jobs(plain_job_mem, score_jobs(segment_rows, true));
        upload_jobs(job_mem, score_jobs(segment_rows, false));
        if (options.graph) {
            check(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal), "beginning capture");
            try {
                enqueue_all(stream);
            } catch (...) {
                cudaGraph_t g = nullptr;
                cudaStreamEndCapture(stream, &g);
                if (g) cudaGraphDestroy(g);
                throw;
            }
            check(cudaStreamEndCapture(stream, &graph), "ending capture");
            check(cudaGraphInstantiate(&graph_exec, graph, 0), "instantiating graph");
        }
        check(cudaStreamSynchronize(stream), "synchronizing");
    }
};

Sweep::Sweep(Executor &executor, const std::vector<Candidate> &owners, const float *frame,
             std::ptrdiff_t frame_stride, const SweepOptions &options)
    : impl_(std::make_unique<Impl>()) {
    if (owners.empty() || !frame) throw std::invalid_argument("a sweep needs candidates and a frame");
    std::vector<std::pair<const AxisPlan *, const AxisPlan *>> candidates;
    for (const auto &[h, v] : owners) candidates.emplace_back(h.get(), v.get());
    const AxisPlan *h0 = candidates.front().first, *v0 = candidates.front().second;
    if (!h0 || !v0) throw std::invalid_argument("sweep candidate without a plan");
    for (const auto &[h, v] : candidates) {
        if (!h || !v || !h->valid() || !v->valid() || h->source_size != h0->source_size
            || v->source_size != v0->source_size)
            throw std::invalid_argument("sweep candidates must share the frame's source size");
    }
    if (frame_stride < h0->source_size) throw std::invalid_argument("invalid frame stride");
    auto &m = *impl_;
    m.executor = &executor;
    m.candidates = candidates;
    m.owners = owners;
    m.frame = frame;
    m.frame_stride = frame_stride;
    m.width = h0->source_size;
    m.height = v0->source_size;
    m.options = options;
    int previous = -1;
    cudaGetDevice(&previous);
    if (previous != executor.device()) check(cudaSetDevice(executor.device()), "selecting device");
    try {
        m.build();
    } catch (...) {
        if (previous >= 0 && previous != executor.device()) cudaSetDevice(previous);
        throw;
    }
    if (previous >= 0 && previous != executor.device()) cudaSetDevice(previous);
}

Sweep::~Sweep() = default;

void Sweep::run(void *stream) {
    auto s = static_cast<cudaStream_t>(stream);
    if (impl_->graph_exec) check(cudaGraphLaunch(impl_->graph_exec, s), "launching sweep graph");
    else impl_->enqueue_all(s);
}

void Sweep::run_plain(void *stream) {
    auto &m = *impl_;
    auto s = static_cast<cudaStream_t>(stream);
    const auto *jobs = reinterpret_cast<const dev::ScoreJob *>(m.plain_job_mem.data());
    for (const auto &w : m.waves) {
        for (int k = 0; k < w.count; ++k) {
            const std::size_t i = static_cast<std::size_t>(w.first + k);
            m.executor->run_batch({w.tasks[static_cast<std::size_t>(k)]}, stream, false);
            if (m.epilogue_of[i] >= 0) {
                check(launch_fused_score_finalize(m.epilogues + m.epilogue_of[i], 1, s), "launching");
            } else {
                const AxisPlan *v = m.candidates[i].second;
                const int col_blocks = m.column_tiles() * m.segments(m.segment_rows);
                int span = 0;
                for (std::size_t q = 0; q < std::size(kSegments); ++q)
                    if (kSegments[q] == m.segment_rows) span = m.spans.at(v)[q];
                const dev::ScoreJob *job = jobs + m.unfused_of[i];
                check(launch_score_tiles(job, 1, col_blocks, span, s), "launching");
                check(launch_score_finalize(job, 1, s), "launching");
            }
            check(cudaStreamSynchronize(s), "synchronizing");
        }
    }
}

std::array<double, 3> Sweep::stage_milliseconds(void *stream) {
    auto &m = *impl_;
    auto s = static_cast<cudaStream_t>(stream);
    std::array<cudaEvent_t, 4> ev{};
    for (auto &e : ev) check(cudaEventCreate(&e), "creating event");
    std::array<double, 3> out{};
    try {
        for (const auto &w : m.waves) {
            check(cudaEventRecord(ev[0], s), "recording event");
            w.batch->launch(s);
            check(cudaEventRecord(ev[1], s), "recording event");
            if (w.unfused)
                check(launch_score_tiles(m.wave_jobs(w), w.unfused, w.column_blocks, m.span_rows(w), s), "launching");
            check(cudaEventRecord(ev[2], s), "recording event");
            if (w.unfused) check(launch_score_finalize(m.wave_jobs(w), w.unfused, s), "launching");
            if (w.fused) check(launch_fused_score_finalize(m.epilogues + w.fused_first, w.fused, s), "launching");
            check(cudaEventRecord(ev[3], s), "recording event");
            check(cudaEventSynchronize(ev[3]), "waiting for event");
            for (int k = 0; k < 3; ++k) {
                float ms = 0.0F;
                check(cudaEventElapsedTime(&ms, ev[static_cast<std::size_t>(k)], ev[static_cast<std::size_t>(k + 1)]),
                      "reading event");
                out[static_cast<std::size_t>(k)] += ms;
            }
        }
    } catch (...) {
        for (auto &e : ev) cudaEventDestroy(e);
        throw;
    }
    for (auto &e : ev) cudaEventDestroy(e);
    return out;
}

void Sweep::read_scores(float *host, void *stream) {
    auto s = static_cast<cudaStream_t>(stream);
    check(cudaMemcpyAsync(host, impl_->score_mem.data(), impl_->candidates.size() * sizeof(float),
                          cudaMemcpyDeviceToHost, s), "reading scores");
    check(cudaStreamSynchronize(s), "synchronizing");
}

const float *Sweep::device_scores() const { return reinterpret_cast<const float *>(impl_->score_mem.data()); }

SweepInfo Sweep::info() const {
    const auto &m = *impl_;
    SweepInfo i;
    i.candidates = static_cast<int>(m.candidates.size());
    i.waves = static_cast<int>(m.waves.size());
    i.device_bytes = m.forward_mem.bytes + m.y_mem.bytes + m.partial_mem.bytes + m.scratch_mem.bytes
        + m.job_mem.bytes + m.plain_job_mem.bytes + m.score_mem.bytes + m.epilogue_mem.bytes;
    for (const auto &w : m.waves)
        i.kernel_launches += w.batch->kernel_launches() + (w.unfused ? 2 : 0) + (w.fused ? 1 : 0);
    i.fused_candidates = m.fused_count;
    i.tune_milliseconds = m.tune_ms;
    i.segment_rows = m.segment_rows;
    i.vectors_per_warp = m.vectors_per_warp ? m.vectors_per_warp : 32;
    i.tuning = m.tuning;
    return i;
}

} // namespace dsmvc_gb
