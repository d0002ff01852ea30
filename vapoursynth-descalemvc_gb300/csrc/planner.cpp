// Host planner: see planner.hpp.  All arithmetic is plain IEEE double with
// no contraction (the build passes -ffp-contract=off), in the operation
// order of the reference planner, src/axis_plan.cpp:246-970.
#include "planner.hpp"

#include "gpu_planner.cuh"

#include <cuda_runtime.h>

#include <algorithm>
#include <bit>
#include <cfloat>
#include <cmath>
#include <atomic>
#include <condition_variable>
#include <cstring>
#include <exception>
#include <limits>
#include <list>
#include <mutex>
#include <numbers>
#include <stdexcept>
#include <string>
#include <thread>
#include <unordered_map>

namespace dsmvc_gb {
namespace {

constexpr double kFloat64Threshold = 1.0e-4;
constexpr double kEps = std::numeric_limits<double>::epsilon();

// ---- kernel weights (src/axis_plan.cpp:246-344) --------------------------

double round_half_up(double v) noexcept {
    return v < 0.0 ? std::floor(v + 0.5) : std::floor(v + 0.49999999999999994);
}
double sq(double v) noexcept { return v * v; }
double cb(double v) noexcept { return v * v * v; }

double sinc(double v) noexcept {
    if (v == 0.0) return 1.0;
    const double s = std::numbers::pi * v;
    return std::sin(s) / s;
}

double kernel_weight(const KernelSpec &k, double distance) noexcept {
    double x = std::abs(distance);
    const double b = k.b, c = k.c;
    switch (k.kind) {
    case KernelKind::bilinear: return std::max(1.0 - x, 0.0);
    case KernelKind::bicubic:
        if (x < 1.0)
            return ((12.0 - 9.0 * b - 6.0 * c) * cb(x)
                    + (-18.0 + 12.0 * b + 6.0 * c) * sq(x) + (6.0 - 2.0 * b)) / 6.0;
        if (x < 2.0)
            return ((-b - 6.0 * c) * cb(x) + (6.0 * b + 30.0 * c) * sq(x)
                    + (-12.0 * b - 48.0 * c) * x + (8.0 * b + 24.0 * c)) / 6.0;
        return 0.0;
    case KernelKind::lanczos:
        return k.taps > 0 && x < static_cast<double>(k.taps)
            ? sinc(x) * sinc(x / static_cast<double>(k.taps)) : 0.0;
    case KernelKind::spline16:
        if (x < 1.0) return 1.0 - x / 5.0 - 9.0 * sq(x) / 5.0 + cb(x);
        if (x < 2.0) { x -= 1.0; return -7.0 * x / 15.0 + 4.0 * sq(x) / 5.0 - cb(x) / 3.0; }
        return 0.0;
    case KernelKind::spline36:
        if (x < 1.0) return 1.0 - 3.0 * x / 209.0 - 453.0 * sq(x) / 209.0 + 13.0 * cb(x) / 11.0;
        if (x < 2.0) { x -= 1.0; return -156.0 * x / 209.0 + 270.0 * sq(x) / 209.0 - 6.0 * cb(x) / 11.0; }
        if (x < 3.0) { x -= 2.0; return 26.0 * x / 209.0 - 45.0 * sq(x) / 209.0 + cb(x) / 11.0; }
        return 0.0;
    case KernelKind::spline64:
        if (x < 1.0) return 1.0 - 3.0 * x / 2911.0 - 6387.0 * sq(x) / 2911.0 + 49.0 * cb(x) / 41.0;
        if (x < 2.0) { x -= 1.0; return -2328.0 * x / 2911.0 + 4032.0 * sq(x) / 2911.0 - 24.0 * cb(x) / 41.0; }
        if (x < 3.0) { x -= 2.0; return 582.0 * x / 2911.0 - 1008.0 * sq(x) / 2911.0 + 6.0 * cb(x) / 41.0; }
        if (x < 4.0) { x -= 3.0; return -97.0 * x / 2911.0 + 168.0 * sq(x) / 2911.0 - cb(x) / 41.0; }
        return 0.0;
    case KernelKind::custom: return 0.0;
    }
    return 0.0;
}

// filter_support (src/axis_plan.cpp:370-424) with its argument checks.
std::int32_t effective_support(const AxisRequest &r) {
    if (r.source_size <= 0 || r.destination_size <= 0)
        throw std::invalid_argument("axis dimensions must be positive");
    if (!(r.active_length > 0.0) || !std::isfinite(r.active_length) || !std::isfinite(r.shift))
        throw std::invalid_argument(
            "active length and shift must be finite, with positive active length");
    if (static_cast<unsigned>(r.border) > 4U) throw std::invalid_argument("padding mode is invalid");
    if (static_cast<unsigned>(r.f64_mode) > 2U) throw std::invalid_argument("f64 mode is invalid");
    if (!(r.kernel.blur > 0.0) || !std::isfinite(r.kernel.blur))
        throw std::invalid_argument("blur must be finite and greater than zero");
    std::int32_t base = 0;
    switch (r.kernel.kind) {
    case KernelKind::bilinear: base = 1; break;
    case KernelKind::bicubic:
    case KernelKind::spline16: base = 2; break;
    case KernelKind::spline36: base = 3; break;
    case KernelKind::spline64: base = 4; break;
    case KernelKind::lanczos:
    case KernelKind::custom: base = r.kernel.taps; break;
    default: throw std::invalid_argument("kernel kind is invalid");
    }
    constexpr auto maximum = (std::numeric_limits<std::int32_t>::max() - 1) / 2;
    if (base <= 0 || base > maximum)
        throw std::invalid_argument("filter support is invalid or too large");
    const double scaled = static_cast<double>(base) * r.kernel.blur;
    if (!std::isfinite(scaled) || scaled > static_cast<double>(maximum))
        throw std::length_error("effective filter support is too large");
    const double support = std::ceil(scaled);
    if (!(support >= 1.0) || support > static_cast<double>(maximum))
        throw std::length_error("effective filter support is too large");
    return static_cast<std::int32_t>(support);
}

struct Csr {
    std::vector<std::uint32_t> offsets;
    std::vector<std::int32_t> indices;
    std::vector<double> weights;
};

// Sampling geometry and the normalised, coalesced descale matrix A
// (src/axis_plan.cpp:456-599): one row per source sample.
Csr descale_matrix(const AxisRequest &r, std::int32_t support, const CustomKernel &custom) {
    const std::int32_t taps = 2 * support;
    const auto cells = static_cast<std::size_t>(r.source_size) * static_cast<std::size_t>(taps);
    if (cells / static_cast<std::size_t>(taps) != static_cast<std::size_t>(r.source_size))
        throw std::length_error("inverse geometry is too large");
    Csr a;
    a.offsets.reserve(static_cast<std::size_t>(r.source_size) + 1U);
    a.indices.reserve(cells);
    a.weights.reserve(cells);
    a.offsets.push_back(0U);
    std::vector<double> distance(static_cast<std::size_t>(taps));
    std::vector<double> weight(static_cast<std::size_t>(taps));
    std::vector<std::int32_t> column(static_cast<std::size_t>(taps));
    std::vector<std::int32_t> unique;
    std::vector<double> merged(static_cast<std::size_t>(taps));
    std::vector<char> used(static_cast<std::size_t>(taps));
    const double ratio = static_cast<double>(r.source_size) / r.active_length;
    const bool unity_blur = r.kernel.blur == 1.0;
    const bool is_custom = r.kernel.kind == KernelKind::custom;
    for (std::int32_t row = 0; row < r.source_size; ++row) {
        const double position = (static_cast<double>(row) + 0.5) / ratio + r.shift;
        const double begin = round_half_up(position - static_cast<double>(support)) + 0.5;
        unique.clear();
        for (std::int32_t t = 0; t < taps; ++t) {
            const double center = begin + static_cast<double>(t);
            distance[t] = center - position;
            const double fl = std::floor(center);
            if (!std::isfinite(fl) || fl < -0x1p63 || fl >= 0x1p63)
                throw std::out_of_range("shift places filter support outside the 64-bit pixel grid");
            const auto idx = padding_index(static_cast<std::int64_t>(fl), r.destination_size, r.border);
            column[t] = idx;
            if (idx >= 0 && std::find(unique.begin(), unique.end(), idx) == unique.end())
                unique.push_back(idx);
        }
        std::sort(unique.begin(), unique.end());
        double total = 0.0;
        for (std::int32_t t = 0; t < taps; ++t) {
            const double d = unity_blur ? distance[t] : distance[t] / r.kernel.blur;
            const double w = is_custom ? custom(std::abs(d)) : kernel_weight(r.kernel, d);
            if (!std::isfinite(w)) throw std::runtime_error("filter returned a non-finite value");
            weight[t] = w;
            total += w;
        }
        if (!std::isfinite(total) || total == 0.0)
            throw std::runtime_error("filter produced a zero or non-finite weight sum");
        const auto count = unique.size();
        std::fill_n(merged.begin(), count, 0.0);
        std::fill_n(used.begin(), count, char{0});
        for (std::int32_t t = 0; t < taps; ++t) {
            if (column[t] < 0) continue;
            const double w = weight[t] / total;
            if (w == 0.0) continue;
            const auto slot = static_cast<std::size_t>(
                std::lower_bound(unique.begin(), unique.end(), column[t]) - unique.begin());
            merged[slot] += w;
            used[slot] = 1;
        }
        for (std::size_t s = 0; s < count; ++s) {
            if (!used[s]) continue;
            a.indices.push_back(unique[s]);
            a.weights.push_back(merged[s]);
        }
        if (a.indices.size() > std::numeric_limits<std::uint32_t>::max())
            throw std::length_error("inverse coefficient table is too large");
        a.offsets.push_back(static_cast<std::uint32_t>(a.indices.size()));
    }
    return a;
}

// Counting-sort transpose (src/axis_plan.cpp:601-626).
Csr transpose(const Csr &a, std::int32_t rows, std::int32_t columns) {
    Csr t;
    t.offsets.assign(static_cast<std::size_t>(columns) + 1U, 0U);
    for (const auto c : a.indices) ++t.offsets[static_cast<std::size_t>(c) + 1U];
    for (std::int32_t c = 0; c < columns; ++c) t.offsets[c + 1] += t.offsets[c];
    t.indices.resize(a.indices.size());
    t.weights.resize(a.weights.size());
    auto cursor = t.offsets;
    for (std::int32_t row = 0; row < rows; ++row) {
        for (auto k = a.offsets[row]; k < a.offsets[row + 1]; ++k) {
            const auto dst = cursor[static_cast<std::size_t>(a.indices[k])]++;
            t.indices[dst] = row;
            t.weights[dst] = a.weights[k];
        }
    }
    return t;
}

// Normal-matrix band (src/axis_plan.cpp:628-668).
std::vector<double> normal_bands(const Csr &t, std::int32_t n, std::int32_t hb) {
    const auto w = static_cast<std::size_t>(n);
    std::vector<double> bands((static_cast<std::size_t>(hb) + 1U) * w, 0.0);
    for (std::int32_t i = 0; i < n; ++i) {
        const auto maxd = std::min(hb, n - i - 1);
        for (std::int32_t d = 0; d <= maxd; ++d) {
            auto l = t.offsets[i], le = t.offsets[i + 1];
            auto r = t.offsets[i + d], re = t.offsets[i + d + 1];
            double sum = 0.0;
            while (l < le && r < re) {
                const auto li = t.indices[l], ri = t.indices[r];
                if (li < ri) ++l;
                else if (ri < li) ++r;
                else { sum += t.weights[l] * t.weights[r]; ++l; ++r; }
            }
            bands[static_cast<std::size_t>(d) * w + static_cast<std::size_t>(i)] = sum;
        }
    }
    return bands;
}

// In-place banded LDL^T (src/axis_plan.cpp:766-791).
void factor_ldlt(std::vector<double> &bands, std::int32_t n, std::int32_t hb) noexcept {
    const auto w = static_cast<std::size_t>(n);
    for (std::int32_t i = 0; i < n; ++i) {
        const auto end = std::min(hb + 1, n - i);
        const double pivot = bands[static_cast<std::size_t>(i)] + kEps;
        for (std::int32_t d = 1; d < end; ++d) {
            const double m = bands[static_cast<std::size_t>(d) * w + static_cast<std::size_t>(i)] / pivot;
            for (std::int32_t o = 0; o < end - d; ++o) {
                bands[static_cast<std::size_t>(o) * w + static_cast<std::size_t>(i + d)] -=
                    m * bands[static_cast<std::size_t>(d + o) * w + static_cast<std::size_t>(i)];
            }
        }
        const double inv = 1.0 / pivot;
        for (std::int32_t d = 1; d < end; ++d)
            bands[static_cast<std::size_t>(d) * w + static_cast<std::size_t>(i)] *= inv;
    }
}

// Banded LDL^T solve used by the Hager estimate (src/axis_plan.cpp:793-823).
void solve_ldlt(const std::vector<double> &f, std::int32_t n, std::int32_t hb, double *v) noexcept {
    const auto w = static_cast<std::size_t>(n);
    for (std::int32_t i = 0; i < n; ++i) {
        double value = v[i];
        for (std::int32_t d = std::min(hb, i); d >= 1; --d)
            value -= f[static_cast<std::size_t>(d) * w + static_cast<std::size_t>(i - d)] * v[i - d];
        v[i] = value;
    }
    for (std::int32_t i = 0; i < n; ++i) v[i] /= f[static_cast<std::size_t>(i)] + kEps;
    for (std::int32_t i = n - 2; i >= 0; --i) {
        double value = v[i];
        for (std::int32_t d = std::min(hb, n - i - 1); d >= 1; --d)
            value -= f[static_cast<std::size_t>(d) * w + static_cast<std::size_t>(i)] * v[i + d];
        v[i] = value;
    }
}

struct Conditioning {
    double rcond = 0.0;
    double one_norm = 0.0;
};

// Three-stage reciprocal condition estimate of the normal matrix
// (src/axis_plan.cpp:675-908): diagonal dominance, then the |L^-1| bound,
// then Hager's 1-norm estimate of G^-1 (at most eight steps).
Conditioning conditioning(const std::vector<double> &g, const std::vector<double> &f,
                          std::int32_t n, std::int32_t hb) {
    const auto w = static_cast<std::size_t>(n);
    std::vector<double> work(w, 0.0);
    for (std::int32_t col = 0; col < n; ++col) {
        work[col] += std::abs(g[static_cast<std::size_t>(col)]);
        for (std::int32_t d = 1, e = std::min(hb, n - col - 1); d <= e; ++d) {
            const double v = std::abs(g[static_cast<std::size_t>(d) * w + static_cast<std::size_t>(col)]);
            work[col] += v;
            work[col + d] += v;
        }
    }
    Conditioning out;
    out.one_norm = *std::max_element(work.begin(), work.end());
    double margin = std::numeric_limits<double>::infinity();
    for (std::int32_t row = 0; row < n; ++row)
        margin = std::min(margin, 2.0 * std::abs(g[static_cast<std::size_t>(row)]) - work[row]);
    out.rcond = margin > 0.0 && out.one_norm > 0.0 ? margin / out.one_norm : 0.0;
    if (out.rcond >= kFloat64Threshold) return out;

    std::fill(work.begin(), work.end(), 1.0);
    double inf_norm = 1.0, diag_norm = 0.0;
    for (std::int32_t row = 0; row < n; ++row) {
        double sum = 1.0;
        for (std::int32_t d = 1, e = std::min(hb, row); d <= e; ++d)
            sum += std::abs(f[static_cast<std::size_t>(d) * w + static_cast<std::size_t>(row - d)]) * work[row - d];
        work[row] = sum;
        inf_norm = std::max(inf_norm, sum);
        diag_norm = std::max(diag_norm, 1.0 / std::abs(f[static_cast<std::size_t>(row)] + kEps));
    }
    std::fill(work.begin(), work.end(), 1.0);
    double one = 1.0;
    for (std::int32_t col = n - 1; col >= 0; --col) {
        double sum = 1.0;
        for (std::int32_t d = 1, e = std::min(hb, n - col - 1); d <= e; ++d)
            sum += std::abs(f[static_cast<std::size_t>(d) * w + static_cast<std::size_t>(col)]) * work[col + d];
        work[col] = sum;
        one = std::max(one, sum);
    }
    const double bound = one * diag_norm * inf_norm;
    if (!(out.one_norm > 0.0) || !(bound > 0.0) || !std::isfinite(out.one_norm) || !std::isfinite(bound))
        out.rcond = 0.0;
    else
        out.rcond = std::clamp(1.0 / (out.one_norm * bound), 0.0, 1.0);
    if (out.rcond >= kFloat64Threshold) return out;

    std::vector<double> x(w, 1.0 / static_cast<double>(n)), y(w), z(w);
    double estimate = 0.0;
    std::size_t previous = w;
    for (int it = 0; it < 8; ++it) {
        y = x;
        solve_ldlt(f, n, hb, y.data());
        double next = 0.0;
        for (const double v : y) next = next + std::abs(v);
        estimate = std::max(estimate, next);
        for (std::size_t i = 0; i < w; ++i) z[i] = y[i] < 0.0 ? -1.0 : 1.0;
        solve_ldlt(f, n, hb, z.data());
        std::size_t index = 0;
        for (std::size_t i = 1; i < w; ++i)
            if (std::abs(z[index]) < std::abs(z[i])) index = i;
        double dot = 0.0;
        for (std::size_t i = 0; i < w; ++i) dot = dot + z[i] * x[i];
        if (index == previous || std::abs(z[index]) <= dot) break;
        std::fill(x.begin(), x.end(), 0.0);
        x[index] = 1.0;
        previous = index;
    }
    if (!(out.one_norm > 0.0) || !(estimate > 0.0) || !std::isfinite(out.one_norm) || !std::isfinite(estimate))
        out.rcond = 0.0;
    else
        out.rcond = std::clamp(1.0 / (out.one_norm * estimate), 0.0, 1.0);
    return out;
}

// ---- single-flight LRU plan cache (src/axis_plan.cpp:110-228) -----------

struct PlanKey {
    std::int32_t source, destination;
    std::uint64_t active, shift;
    KernelKind kind;
    std::int32_t taps;
    std::uint64_t b, c, blur;
    BorderMode border;
    F64Mode mode;
    bool operator==(const PlanKey &) const = default;
};

struct PlanKeyHash {
    std::size_t operator()(const PlanKey &k) const noexcept {
        std::uint64_t h = 1469598103934665603ULL;
        auto mix = [&h](std::uint64_t v) { h ^= v; h *= 1099511628211ULL; };
        mix(static_cast<std::uint32_t>(k.source));
        mix(static_cast<std::uint32_t>(k.destination));
        mix(k.active);
        mix(k.shift);
        mix(static_cast<std::uint8_t>(k.kind));
        mix(static_cast<std::uint32_t>(k.taps));
        mix(k.b);
        mix(k.c);
        mix(k.blur);
        mix(static_cast<std::uint8_t>(k.mode));
        mix(static_cast<std::uint8_t>(k.border));
        return static_cast<std::size_t>(h);
    }
};

PlanKey key_of(const AxisRequest &r) noexcept {
    const bool bicubic = r.kernel.kind == KernelKind::bicubic;
    return {r.source_size, r.destination_size,
            std::bit_cast<std::uint64_t>(r.active_length), std::bit_cast<std::uint64_t>(r.shift),
            r.kernel.kind, r.kernel.kind == KernelKind::lanczos ? r.kernel.taps : 0,
            bicubic ? std::bit_cast<std::uint64_t>(r.kernel.b) : 0U,
            bicubic ? std::bit_cast<std::uint64_t>(r.kernel.c) : 0U,
            std::bit_cast<std::uint64_t>(r.kernel.blur), r.border, r.f64_mode};
}

class PlanCache {
    struct Entry {
        std::shared_ptr<const AxisPlan> value;
        std::exception_ptr error;
        bool ready = false;
        bool resident = false;
        std::size_t bytes = 0;
        std::list<PlanKey>::iterator position;
        std::condition_variable changed;
    };

public:
    std::shared_ptr<const AxisPlan> get(const AxisRequest &request) {
        const auto key = key_of(request);
        std::shared_ptr<Entry> entry;
        {
            std::unique_lock lock(mutex_);
            if (auto it = map_.find(key); it != map_.end()) {
                entry = it->second;
                entry->changed.wait(lock, [&] { return entry->ready; });
                if (entry->error) std::rethrow_exception(entry->error);
                ++hits_;
                if (entry->resident) lru_.splice(lru_.begin(), lru_, entry->position);
                return entry->value;
            }
            entry = std::make_shared<Entry>();
            map_.emplace(key, entry);
        }
        std::shared_ptr<const AxisPlan> value;
        try {
            value = std::make_shared<const AxisPlan>(build_axis_plan(request));
        } catch (...) {
            {
                std::scoped_lock lock(mutex_);
                entry->error = std::current_exception();
                entry->ready = true;
                if (auto it = map_.find(key); it != map_.end() && it->second == entry) map_.erase(it);
            }
            entry->changed.notify_all();
            throw;
        }
        {
            std::scoped_lock lock(mutex_);
            entry->value = value;
            entry->bytes = value->storage_bytes();
            entry->ready = true;
            auto it = map_.find(key);
            const bool current = it != map_.end() && it->second == entry;
            if (current && entry->bytes <= kMaxBytes) {
                lru_.push_front(key);
                entry->position = lru_.begin();
                entry->resident = true;
                bytes_ += entry->bytes;
                while (lru_.size() > kMaxEntries || bytes_ > kMaxBytes) {
                    auto victim = map_.find(lru_.back());
                    lru_.pop_back();
                    if (victim == map_.end()) continue;
                    bytes_ -= victim->second->bytes;
                    victim->second->resident = false;
                    map_.erase(victim);
                }
            } else if (current) {
                map_.erase(it);
            }
        }
        entry->changed.notify_all();
        return value;
    }

    PlannerCacheStats stats() {
        std::scoped_lock lock(mutex_);
        PlannerCacheStats s;
        s.plan_hits = hits_;
        s.plan_entries = lru_.size();
        s.plan_resident_bytes = bytes_;
        return s;
    }

    void clear() {
        std::scoped_lock lock(mutex_);
        map_.clear();
        lru_.clear();
        bytes_ = 0;
        hits_ = 0;
    }

private:
    static constexpr std::size_t kMaxEntries = 2048;
    static constexpr std::size_t kMaxBytes = 256U << 20;
    std::mutex mutex_;
    std::unordered_map<PlanKey, std::shared_ptr<Entry>, PlanKeyHash> map_;
    std::list<PlanKey> lru_;
    std::size_t bytes_ = 0;
    std::uint64_t hits_ = 0;
};

PlanCache &cache() {
    static PlanCache instance;
    return instance;
}

std::atomic<std::uint64_t> g_builds{0};

// FNV-1a stream of tests/numerical_conformance.hpp:22-80.
struct Fnv {
    std::uint64_t v = 1469598103934665603ULL;
    void byte(std::uint8_t b) { v ^= b; v *= 1099511628211ULL; }
    void u(std::uint64_t x, int n) { for (int i = 0; i < n; ++i) { byte(static_cast<std::uint8_t>(x)); x >>= 8; } }
    void str(const char *s) { const auto n = std::strlen(s); u(n, 8); for (std::size_t i = 0; i < n; ++i) byte(static_cast<std::uint8_t>(s[i])); }
    void f64(double d) { u(std::bit_cast<std::uint64_t>(d), 8); }
    void f32(float f) { u(std::bit_cast<std::uint32_t>(f), 4); }
    void i32(std::int32_t i) { u(static_cast<std::uint32_t>(i), 4); }
    template <class T> void span(const std::vector<T> &values) {
        u(values.size(), 8);
        for (const T x : values) {
            if constexpr (std::is_same_v<T, float>) f32(x);
            else if constexpr (std::is_same_v<T, double>) f64(x);
            else u(static_cast<std::uint64_t>(static_cast<std::make_unsigned_t<T>>(x)), sizeof(T));
        }
    }
    void head(const AxisRequest &r, const AxisPlan &p) {
        i32(r.source_size); i32(r.destination_size); f64(r.active_length); f64(r.shift);
        u(static_cast<std::uint8_t>(r.kernel.kind), 1); i32(r.kernel.taps); f64(r.kernel.b); f64(r.kernel.c);
        u(static_cast<std::uint8_t>(r.border), 1); u(static_cast<std::uint8_t>(r.f64_mode), 1);
        i32(p.source_size); i32(p.destination_size); i32(p.support); i32(p.half_bandwidth);
        f64(p.active_length); f64(p.shift);
    }
    void f32_arrays(const AxisPlan &p) {
        span(p.transpose_offsets); span(p.transpose_indices); span(p.transpose_weights);
        span(p.lower_ld); span(p.upper_l); span(p.inverse_diagonal);
    }
};

} // namespace

std::int32_t padding_index(std::int64_t index, std::int32_t size, BorderMode mode) {
    if (size <= 0) throw std::invalid_argument("padding size must be positive");
    if (static_cast<unsigned>(mode) > 4U) throw std::invalid_argument("padding mode is invalid");
    const auto extent = static_cast<std::int64_t>(size);
    if (index >= 0 && index < extent) return static_cast<std::int32_t>(index);
    switch (mode) {
    case BorderMode::zero: return -1;
    case BorderMode::repeat: return index < 0 ? 0 : size - 1;
    case BorderMode::reflect101: {
        if (size == 1) return 0;
        const auto period = 2 * (extent - 1);
        auto m = index % period;
        if (m < 0) m += period;
        return static_cast<std::int32_t>(m < extent ? m : period - m);
    }
    case BorderMode::symmetric: {
        const auto period = 2 * extent;
        auto m = index % period;
        if (m < 0) m += period;
        return static_cast<std::int32_t>(m < extent ? m : period - 1 - m);
    }
    case BorderMode::mirror:
        if (index < -extent || index >= 2 * extent) return -1;
        return static_cast<std::int32_t>(index < 0 ? -index - 1 : 2 * extent - index - 1);
    }
    throw std::invalid_argument("padding mode is invalid");
}

std::size_t AxisPlan::storage_bytes() const noexcept {
    return sizeof(*this) + transpose_offsets.capacity() * 4 + transpose_indices.capacity() * 4
        + transpose_weights.capacity() * 4 + lower_ld.capacity() * 4 + upper_l.capacity() * 4
        + inverse_diagonal.capacity() * 4 + transpose_weights_f64.capacity() * 8
        + normal_bands_f64.capacity() * 8 + ldlt_bands_f64.capacity() * 8
        + inverse_diagonal_f64.capacity() * 8;
}

bool AxisPlan::valid() const noexcept {
    if (validated) return true;
    if (source_size <= 0 || destination_size <= 0 || support <= 0 || half_bandwidth < 0
        || half_bandwidth >= destination_size || !(active_length > 0.0)
        || !std::isfinite(active_length) || !std::isfinite(shift) || !std::isfinite(normal_rcond)
        || normal_rcond < 0.0 || normal_rcond > 1.0 || !std::isfinite(normal_inf_norm)
        || normal_inf_norm < 0.0)
        return false;
    const auto n = static_cast<std::size_t>(destination_size);
    const auto factors = static_cast<std::size_t>(half_bandwidth) * n;
    if (transpose_offsets.size() != n + 1U || transpose_indices.size() != transpose_weights.size()
        || transpose_offsets.front() != 0U || transpose_offsets.back() != transpose_indices.size()
        || lower_ld.size() != factors || upper_l.size() != factors || inverse_diagonal.size() != n)
        return false;
    const bool f64 = !ldlt_bands_f64.empty();
    if (f64 != !transpose_weights_f64.empty() || f64 != !normal_bands_f64.empty()
        || f64 != !inverse_diagonal_f64.empty())
        return false;
    if (f64 ? !(normal_inf_norm > 0.0) : normal_inf_norm != 0.0) return false;
    const auto bands = (static_cast<std::size_t>(half_bandwidth) + 1U) * n;
    if (f64 && (transpose_weights_f64.size() != transpose_weights.size()
                || normal_bands_f64.size() != bands || ldlt_bands_f64.size() != bands
                || inverse_diagonal_f64.size() != n))
        return false;
    for (std::size_t row = 0; row < n; ++row) {
        const auto b = transpose_offsets[row], e = transpose_offsets[row + 1];
        if (b > e || e > transpose_indices.size()) return false;
        std::int32_t previous = -1;
        for (auto k = b; k < e; ++k) {
            const auto s = transpose_indices[k];
            if (s < 0 || s >= source_size || s <= previous || !std::isfinite(transpose_weights[k]))
                return false;
            previous = s;
        }
    }
    auto finite = [](const auto &v) {
        return std::all_of(v.begin(), v.end(), [](auto x) { return std::isfinite(x); });
    };
    if (!finite(lower_ld) || !finite(upper_l) || !finite(inverse_diagonal)) return false;
    return !f64 || (finite(transpose_weights_f64) && finite(normal_bands_f64)
                    && finite(ldlt_bands_f64) && finite(inverse_diagonal_f64));
}

AxisPlan build_axis_plan(const AxisRequest &request, const CustomKernel &custom) {
    g_builds.fetch_add(1U, std::memory_order_relaxed);
    const auto support = effective_support(request);
    if (request.kernel.kind == KernelKind::custom && !custom)
        throw std::invalid_argument("custom kernel callback is missing");
    const auto n = request.destination_size;
    const auto w = static_cast<std::size_t>(n);
    auto t = transpose(descale_matrix(request, support, custom), request.source_size, n);
    const auto hb = std::min(2 * support - 1, n - 1);
    auto g = normal_bands(t, n, hb);
    auto f = g;
    factor_ldlt(f, n, hb);
    const auto cond = conditioning(g, f, n, hb);
    const bool f64 = request.f64_mode == F64Mode::float64_only
        || (request.f64_mode == F64Mode::automatic && cond.rcond < kFloat64Threshold);

    AxisPlan p;
    p.source_size = request.source_size;
    p.destination_size = n;
    p.support = support;
    p.half_bandwidth = hb;
    p.active_length = request.active_length;
    p.shift = request.shift;
    p.normal_rcond = cond.rcond;
    p.transpose_weights.resize(t.weights.size());
    std::transform(t.weights.begin(), t.weights.end(), p.transpose_weights.begin(),
                   [](double x) { return static_cast<float>(x); });
    for (std::int32_t i = 0; i < n; ++i)
        p.max_row_entries = std::max<std::int32_t>(
            p.max_row_entries, static_cast<std::int32_t>(t.offsets[i + 1] - t.offsets[i]));
    if (f64) {
        p.normal_inf_norm = cond.one_norm;
        p.transpose_weights_f64 = t.weights;
        p.normal_bands_f64 = g;
        p.ldlt_bands_f64 = f;
        p.inverse_diagonal_f64.resize(w);
        for (std::int32_t i = 0; i < n; ++i) p.inverse_diagonal_f64[i] = 1.0 / (f[i] + kEps);
    }
    p.transpose_offsets = std::move(t.offsets);
    p.transpose_indices = std::move(t.indices);
    p.lower_ld.assign(static_cast<std::size_t>(hb) * w, 0.0F);
    p.upper_l.assign(static_cast<std::size_t>(hb) * w, 0.0F);
    p.inverse_diagonal.resize(w);
    for (std::int32_t i = 0; i < n; ++i) {
        const double diagonal = f[static_cast<std::size_t>(i)];
        p.inverse_diagonal[i] = static_cast<float>(1.0 / (diagonal + kEps));
        for (std::int32_t d = 1, e = std::min(hb, n - i - 1); d <= e; ++d) {
            const double l = f[static_cast<std::size_t>(d) * w + static_cast<std::size_t>(i)];
            p.upper_l[static_cast<std::size_t>(d - 1) * w + static_cast<std::size_t>(i)] = static_cast<float>(l);
            p.lower_ld[static_cast<std::size_t>(d - 1) * w + static_cast<std::size_t>(i + d)] =
                static_cast<float>(l * diagonal);
        }
    }
    if (!p.valid()) throw std::runtime_error("failed to build inverse axis plan");
    p.validated = true;
    return p;
}

std::shared_ptr<const AxisPlan> get_or_build_axis_plan(const AxisRequest &request,
                                                       const CustomKernel &custom) {
    if (request.kernel.kind == KernelKind::custom)
        return std::make_shared<const AxisPlan>(build_axis_plan(request, custom));
    return cache().get(request);
}

PlannerCacheStats planner_cache_stats() {
    auto s = cache().stats();
    s.plan_builds = g_builds.load(std::memory_order_relaxed);
    return s;
}

void clear_planner_caches() {
    cache().clear();
    g_builds.store(0, std::memory_order_relaxed);
}

std::uint64_t f32_plan_hash(const AxisRequest &r, const AxisPlan &p) {
    Fnv h;
    h.str("dsmvc-f32-axis-plan-v1");
    h.head(r, p);
    h.u(p.normal_rcond < 1.0e-4 ? 1 : 0, 1);
    h.u(p.requires_float64() ? 1 : 0, 1);
    h.f32_arrays(p);
    return h.v;
}

std::uint64_t complete_plan_hash(const AxisRequest &r, const AxisPlan &p) {
    Fnv h;
    h.str("dsmvc-axis-plan-v1");
    h.head(r, p);
    h.f64(p.normal_rcond);
    h.f64(p.normal_inf_norm);
    h.f32_arrays(p);
    h.span(p.transpose_weights_f64);
    h.span(p.normal_bands_f64);
    h.span(p.ldlt_bands_f64);
    h.span(p.inverse_diagonal_f64);
    return h.v;
}

// ---- device planning batch ------------------------------------------------

namespace {

void device_check(cudaError_t e, const char *what) {
    if (e != cudaSuccess) throw std::runtime_error(std::string("CUDA ") + what + ": " + cudaGetErrorString(e));
}

struct HostHalf {
    std::int32_t support = 0;
    std::int32_t hb = 0;
    Csr t;
};

// One batch of at most 65535 plans.
void plan_batch_on_device(const AxisRequest *requests, HostHalf *halves, std::size_t count, AxisPlan *out) {
    std::vector<PlannerJob> jobs(count);
    std::int64_t offsets = 0, entries = 0, bands = 0, factors = 0, diagonal = 0, work = 0;
    int max_n = 1;
    for (std::size_t k = 0; k < count; ++k) {
        const auto &h = halves[k];
        auto &j = jobs[k];
        j.n = requests[k].destination_size;
        j.hb = h.hb;
        j.mode = static_cast<std::int32_t>(requests[k].f64_mode);
        j.offsets_at = offsets;
        j.entries_at = entries;
        j.bands_at = bands;
        j.factors_at = factors;
        j.diagonal_at = diagonal;
        j.work_at = work;
        offsets += j.n + 1;
        entries += static_cast<std::int64_t>(h.t.indices.size());
        bands += static_cast<std::int64_t>(h.hb + 1) * j.n;
        factors += static_cast<std::int64_t>(h.hb) * j.n;
        diagonal += j.n;
        work += 4 * static_cast<std::int64_t>(j.n);
        max_n = std::max(max_n, j.n);
    }
    // One device allocation: inputs first (one upload), then the outputs.
    auto al = [](std::size_t v) { return (v + 255) / 256 * 256; };
    const std::size_t b_jobs = al(count * sizeof(PlannerJob)), b_off = al(static_cast<std::size_t>(offsets) * 4),
                      b_idx = al(static_cast<std::size_t>(entries) * 4), b_w = al(static_cast<std::size_t>(entries) * 8);
    const std::size_t in_bytes = b_jobs + b_off + b_idx + b_w;
    const std::size_t b_bands = al(static_cast<std::size_t>(bands) * 8), b_fac = al(static_cast<std::size_t>(factors) * 4),
                      b_diag = al(static_cast<std::size_t>(diagonal) * 4), b_diag64 = al(static_cast<std::size_t>(diagonal) * 8),
                      b_work = al(static_cast<std::size_t>(work) * 8), b_res = al(count * sizeof(PlannerResult));
    const std::size_t total = in_bytes + 2 * b_bands + 2 * b_fac + b_diag + b_diag64 + b_work + b_res;
    std::vector<char> host(in_bytes, 0);
    std::memcpy(host.data(), jobs.data(), count * sizeof(PlannerJob));
    {
        char *o = host.data() + b_jobs;
        char *ix = o + b_off;
        char *w = ix + b_idx;
        for (std::size_t k = 0; k < count; ++k) {
            const auto &t = halves[k].t;
            std::memcpy(o + jobs[k].offsets_at * 4, t.offsets.data(), t.offsets.size() * 4);
            std::memcpy(ix + jobs[k].entries_at * 4, t.indices.data(), t.indices.size() * 4);
            std::memcpy(w + jobs[k].entries_at * 8, t.weights.data(), t.weights.size() * 8);
        }
    }
    char *dev = nullptr;
    device_check(cudaMalloc(&dev, total), "allocating the planning batch");
    struct Free {
        char *p;
        ~Free() { cudaFree(p); }
    } release{dev};
    cudaStream_t stream = nullptr;
    device_check(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "creating a stream");
    struct Destroy {
        cudaStream_t s;
        ~Destroy() { cudaStreamDestroy(s); }
    } destroy{stream};
    device_check(cudaMemcpyAsync(dev, host.data(), in_bytes, cudaMemcpyHostToDevice, stream), "uploading plans");
    PlannerBatch b;
    b.jobs = reinterpret_cast<const PlannerJob *>(dev);
    b.count = static_cast<int>(count);
    b.max_n = max_n;
    b.offsets = reinterpret_cast<const std::uint32_t *>(dev + b_jobs);
    b.indices = reinterpret_cast<const std::int32_t *>(dev + b_jobs + b_off);
    b.weights = reinterpret_cast<const double *>(dev + b_jobs + b_off + b_idx);
    char *o = dev + in_bytes;
    b.bands = reinterpret_cast<double *>(o);
    b.factor = reinterpret_cast<double *>(o + b_bands);
    b.lower = reinterpret_cast<float *>(o + 2 * b_bands);
    b.upper = reinterpret_cast<float *>(o + 2 * b_bands + b_fac);
    b.inv_diag = reinterpret_cast<float *>(o + 2 * b_bands + 2 * b_fac);
    b.inv_diag64 = reinterpret_cast<double *>(o + 2 * b_bands + 2 * b_fac + b_diag);
    b.work = reinterpret_cast<double *>(o + 2 * b_bands + 2 * b_fac + b_diag + b_diag64);
    b.results = reinterpret_cast<PlannerResult *>(o + 2 * b_bands + 2 * b_fac + b_diag + b_diag64 + b_work);
    device_check(static_cast<cudaError_t>(launch_device_planner(b, stream)), "launching the device planner");
    // Float32 arrays and results of every plan in three copies.
    std::vector<float> lower(static_cast<std::size_t>(factors)), upper(static_cast<std::size_t>(factors)),
        inv(static_cast<std::size_t>(diagonal));
    std::vector<PlannerResult> results(count);
    device_check(cudaMemcpyAsync(lower.data(), b.lower, lower.size() * 4, cudaMemcpyDeviceToHost, stream), "reading plans");
    device_check(cudaMemcpyAsync(upper.data(), b.upper, upper.size() * 4, cudaMemcpyDeviceToHost, stream), "reading plans");
    device_check(cudaMemcpyAsync(inv.data(), b.inv_diag, inv.size() * 4, cudaMemcpyDeviceToHost, stream), "reading plans");
    device_check(cudaMemcpyAsync(results.data(), b.results, count * sizeof(PlannerResult), cudaMemcpyDeviceToHost, stream),
                 "reading plans");
    device_check(cudaStreamSynchronize(stream), "planning on the device");
    for (std::size_t k = 0; k < count; ++k) {
        const auto &r = requests[k];
        auto &h = halves[k];
        const auto &res = results[k];
        const auto n = r.destination_size;
        const auto w = static_cast<std::size_t>(n);
        AxisPlan &p = out[k];
        p.source_size = r.source_size;
        p.destination_size = n;
        p.support = h.support;
        p.half_bandwidth = h.hb;
        p.active_length = r.active_length;
        p.shift = r.shift;
        p.normal_rcond = res.rcond;
        p.transpose_weights.resize(h.t.weights.size());
        std::transform(h.t.weights.begin(), h.t.weights.end(), p.transpose_weights.begin(),
                       [](double x) { return static_cast<float>(x); });
        for (std::int32_t i = 0; i < n; ++i)
            p.max_row_entries = std::max<std::int32_t>(
                p.max_row_entries, static_cast<std::int32_t>(h.t.offsets[i + 1] - h.t.offsets[i]));
        if (res.f64) {
            const std::size_t nb = (static_cast<std::size_t>(h.hb) + 1U) * w;
            p.normal_inf_norm = res.one_norm;
            p.normal_bands_f64.resize(nb);
            p.ldlt_bands_f64.resize(nb);
            p.inverse_diagonal_f64.resize(w);
            device_check(cudaMemcpyAsync(p.normal_bands_f64.data(), b.bands + jobs[k].bands_at, nb * 8,
                                         cudaMemcpyDeviceToHost, stream), "reading plans");
            device_check(cudaMemcpyAsync(p.ldlt_bands_f64.data(), b.factor + jobs[k].bands_at, nb * 8,
                                         cudaMemcpyDeviceToHost, stream), "reading plans");
            device_check(cudaMemcpyAsync(p.inverse_diagonal_f64.data(), b.inv_diag64 + jobs[k].diagonal_at, w * 8,
                                         cudaMemcpyDeviceToHost, stream), "reading plans");
            p.transpose_weights_f64 = h.t.weights;
        }
        p.transpose_offsets = std::move(h.t.offsets);
        p.transpose_indices = std::move(h.t.indices);
        const auto f_at = static_cast<std::size_t>(jobs[k].factors_at);
        const auto d_at = static_cast<std::size_t>(jobs[k].diagonal_at);
        p.lower_ld.assign(lower.begin() + static_cast<std::ptrdiff_t>(f_at),
                          lower.begin() + static_cast<std::ptrdiff_t>(f_at + static_cast<std::size_t>(h.hb) * w));
        p.upper_l.assign(upper.begin() + static_cast<std::ptrdiff_t>(f_at),
                         upper.begin() + static_cast<std::ptrdiff_t>(f_at + static_cast<std::size_t>(h.hb) * w));
        p.inverse_diagonal.assign(inv.begin() + static_cast<std::ptrdiff_t>(d_at),
                                  inv.begin() + static_cast<std::ptrdiff_t>(d_at + w));
    }
    device_check(cudaStreamSynchronize(stream), "reading Float64 plans");
    for (std::size_t k = 0; k < count; ++k) {
        if (!out[k].valid()) throw std::runtime_error("failed to build inverse axis plan");
        out[k].validated = true;
    }
}

} // namespace

std::vector<AxisPlan> build_axis_plans_on_device(const std::vector<AxisRequest> &requests, int device,
                                                 int threads) {
    const std::size_t count = requests.size();
    std::vector<AxisPlan> out(count);
    if (count == 0) return out;
    for (const auto &r : requests)
        if (r.kernel.kind == KernelKind::custom)
            throw std::invalid_argument("custom kernels are planned on the host (build_axis_plan)");
    g_builds.fetch_add(count, std::memory_order_relaxed);
    // The host half (geometry, kernel weights, the A^T CSR) on host threads.
    std::vector<HostHalf> halves(count);
    std::vector<std::string> errors(count);
    std::atomic<std::size_t> next{0};
    auto worker = [&] {
        for (std::size_t i = next++; i < count; i = next++) {
            try {
                const auto &r = requests[i];
                auto &h = halves[i];
                h.support = effective_support(r);
                h.t = transpose(descale_matrix(r, h.support, {}), r.source_size, r.destination_size);
                h.hb = std::min(2 * h.support - 1, r.destination_size - 1);
            } catch (const std::exception &e) {
                errors[i] = e.what();
            }
        }
    };
    unsigned n = threads > 0 ? static_cast<unsigned>(threads) : std::thread::hardware_concurrency();
    n = std::max(1U, std::min<unsigned>(n, static_cast<unsigned>(count)));
    std::vector<std::thread> pool;
    for (unsigned t = 1; t < n; ++t) pool.emplace_back(worker);
    worker();
    for (auto &t : pool) t.join();
    for (std::size_t i = 0; i < count; ++i)
        if (!errors[i].empty()) throw std::invalid_argument("plan " + std::to_string(i) + ": " + errors[i]);

    int previous = -1;
    device_check(cudaGetDevice(&previous), "querying the device");
    if (device >= 0) device_check(cudaSetDevice(device), "selecting the device");
    struct Restore {
        int d;
        ~Restore() { if (d >= 0) cudaSetDevice(d); }
    } restore{previous};
    constexpr std::size_t kBatch = 65535;
    for (std::size_t at = 0; at < count; at += kBatch)
        plan_batch_on_device(requests.data() + at, halves.data() + at, std::min(kBatch, count - at), out.data() + at);
    return out;
}

} // namespace dsmvc_gb
