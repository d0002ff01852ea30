// Streaming-kernel packing (see stream_plan.hpp).
#include "stream_plan.hpp"

#include "stream.cuh"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>

namespace dsmvc_gb {
namespace {

int round4(int v) { return (v + 3) / 4 * 4; }

// Simulates the kernel's ring feeder: loads of `granule` samples while they
// fit in the vector, single samples at the tail.  True when every window is
// still resident when its destination is computed.
bool ring_fits(const std::vector<int> &s0, int window, int size, int granule, int ring) {
    int have = 0;
    for (const int start : s0) {
        const int need = start + window;
        while (have < need) have += (have + granule <= size) ? granule : 1;
        if (have - start > ring) return false;
    }
    return true;
}

// The transposing kernels feed a warp's ring in blocks of 16 samples once
// per group of 4 destinations (up to the window end of the group's last
// destination, single samples past the last whole block).  True when every
// destination's window is still resident.
bool ring_fits_grouped(const std::vector<int> &s0, int window, int size, int ring) {
    int have = 0;
    const int n = static_cast<int>(s0.size());
    for (int g = 0; g < n; g += 4) {
        const int last = std::min(g + 3, n - 1);
        const int need = std::min(size, std::max(s0[g], s0[last]) + window);
        while (have < need) have += (have + 16 <= size) ? 16 : 1;
        for (int j = g; j <= last; ++j)
            if (have - s0[j] > ring) return false;
    }
    return true;
}

} // namespace

StreamPack pack_stream_plan(const AxisPlan &p, int chunk, int ring, bool hb_supported, bool hb_supported_exact) {
    StreamPack out;
    const int n = p.destination_size, m = p.source_size, hb = p.half_bandwidth;
    if (!hb_supported && !hb_supported_exact) {
        out.reason = "half-bandwidth without a streaming kernel";
        return out;
    }
    if (p.requires_float64()) {
        out.reason = "Float64 plan";
        return out;
    }
    // Dense window: widest span of sources feeding one destination.
    int span = 1;
    for (int j = 0; j < n; ++j) {
        const auto b = p.transpose_offsets[j], e = p.transpose_offsets[j + 1];
        if (b < e) span = std::max(span, p.transpose_indices[e - 1] - p.transpose_indices[b] + 1);
    }
    const int window = round4(span);
    if (window > m || window > ring) {
        out.reason = "gather window exceeds the source or the ring";
        return out;
    }
    std::vector<int> s0(static_cast<std::size_t>(n));
    int previous = 0;
    for (int j = 0; j < n; ++j) {
        const auto b = p.transpose_offsets[j], e = p.transpose_offsets[j + 1];
        int first = b < e ? p.transpose_indices[b] : previous;
        first = std::min(first, m - window);
        if (first < previous) {
            out.reason = "gather windows move backwards";
            return out;
        }
        s0[j] = first;
        previous = first;
    }
    out.ring_ok_f32 = ring_fits(s0, window, m, 4, ring);
    out.ring_ok_u16 = ring_fits(s0, window, m, 8, ring);
    out.ring_ok_u8 = ring_fits(s0, window, m, 16, ring);
    // The transposing kernels keep the ring's first 16 rows twice: windows of
    // up to 16 samples.
    out.ring_ok_transposed = ring_fits_grouped(s0, window, m, ring) && window <= 16;
    // The two-pass transposing kernels refill their ring per destination in
    // blocks of 16 (per group of four destinations with window 8 when the
    // grouped replay holds).
    out.exact = hb_supported_exact && out.ring_ok_u8 && window <= 16;
    if (!out.ring_ok_f32) out.reason = "gather windows advance faster than the ring";
    else if (!hb_supported) out.reason = "half-bandwidth without a chunk-delayed kernel";

    // Backward warm-up accuracy: the carry entering a chunk's end, pushed
    // through the chunk's homogeneous backward recurrence, must vanish.
    const auto w = static_cast<std::size_t>(n);
    const int chunks = (n + chunk - 1) / chunk;
    double worst = 0.0;
    std::vector<double> x(static_cast<std::size_t>(chunk + hb));
    for (int k = 1; k + 1 < chunks; ++k) {           // chunks that serve as warm-up
        const int lo = k * chunk, hi = lo + chunk;     // full chunk [lo, hi)
        for (int e = 0; e < hb; ++e) {
            std::fill(x.begin(), x.end(), 0.0);
            x[static_cast<std::size_t>(chunk + e)] = 1.0; // unit carry at x_{hi+e}
            for (int t = hi - 1; t >= lo; --t) {
                double s = 0.0;
                for (int d = 1; d <= hb && t + d < n; ++d) {
                    s += static_cast<double>(p.upper_l[static_cast<std::size_t>(d - 1) * w + static_cast<std::size_t>(t)])
                        * x[static_cast<std::size_t>(t + d - lo)];
                }
                x[static_cast<std::size_t>(t - lo)] = -s;
            }
            for (int q = 0; q < hb; ++q) worst = std::max(worst, std::abs(x[static_cast<std::size_t>(q)]));
        }
    }
    out.backward_transfer = worst;
    if (out.reason.empty() && !(worst <= std::ldexp(1.0, -26)))
        out.reason = "backward carry decays too slowly for one chunk";

    // Forward warm-up accuracy for segments: a unit history entering chunk k
    // (y_{lo-1-e} = 1), pushed through the chunk's homogeneous forward
    // recurrence y_t = -inv_t * sum_d lower_ld(d, t) y_{t-d}, must vanish.
    // Chunk 0 needs no check (its history is the true, empty one).
    double fworst = 0.0;
    for (int k = 1; k + 1 < chunks; ++k) {
        const int lo = k * chunk, hi = lo + chunk;
        for (int e = 0; e < hb; ++e) {
            std::fill(x.begin(), x.end(), 0.0);
            x[static_cast<std::size_t>(hb - 1 - e)] = 1.0;  // x[i] holds y_{lo - hb + i}
            for (int t = lo; t < hi; ++t) {
                double s = 0.0;
                for (int d = 1; d <= hb && d <= t; ++d)
                    s += static_cast<double>(p.lower_ld[static_cast<std::size_t>(d - 1) * w + static_cast<std::size_t>(t)])
                        * x[static_cast<std::size_t>(t - d - lo + hb)];
                x[static_cast<std::size_t>(t - lo + hb)] = -s * static_cast<double>(p.inverse_diagonal[static_cast<std::size_t>(t)]);
            }
            for (int q = 0; q < hb; ++q)
                fworst = std::max(fworst, std::abs(x[static_cast<std::size_t>(chunk + q)]));
        }
    }
    out.forward_transfer = fworst;
    const bool delayed = out.reason.empty();
    if (!delayed && !out.exact) return out;

    const int low = round4(hb);
    out.window = window;
    out.forward_stride = 4 + window + low;
    out.backward_stride = std::max(4, low);
    // Whole chunks of records, so that every chunk copy of the kernel stays
    // inside the arrays.  Records past the last destination are zero except
    // for their window start, which repeats the last destination's: the
    // kernels size each ring refill by the window starts of a group's first
    // and last records, and a padding record must not hide the windows of
    // the valid destinations before it in its group.
    const auto padded = static_cast<std::size_t>((n + chunk - 1) / chunk) * static_cast<std::size_t>(chunk);
    out.forward.assign(padded * static_cast<std::size_t>(out.forward_stride), 0.0F);
    out.backward.assign(padded * static_cast<std::size_t>(out.backward_stride), 0.0F);
    // Word 2 of a forward record: the window's offset in the transposing
    // kernels' ring, (s0 mod 32) * kTRingPitch.
    auto header = [&](float *f, int start) {
        const int ring_offset = (start & (kStreamRing - 1)) * kTRingPitch;
        std::memcpy(&f[0], &start, sizeof(int));
        std::memcpy(&f[2], &ring_offset, sizeof(int));
    };
    for (std::size_t j = static_cast<std::size_t>(n); j < padded; ++j)
        header(&out.forward[j * static_cast<std::size_t>(out.forward_stride)], s0.back());
    for (int j = 0; j < n; ++j) {
        float *f = out.forward.data() + static_cast<std::size_t>(j) * out.forward_stride;
        header(f, s0[j]);
        f[1] = p.inverse_diagonal[j];
        for (auto k = p.transpose_offsets[j]; k < p.transpose_offsets[j + 1]; ++k)
            f[4 + (p.transpose_indices[k] - s0[j])] = p.transpose_weights[k];
        for (int q = 0; q < hb; ++q) {
            const int d = hb - q;                      // use order d = hb..1
            f[4 + window + q] = d <= j
                ? -p.lower_ld[static_cast<std::size_t>(d - 1) * w + static_cast<std::size_t>(j)] : 0.0F;
        }
        float *b = out.backward.data() + static_cast<std::size_t>(j) * out.backward_stride;
        const int avail = std::min(hb, n - j - 1);
        for (int q = 0; q < hb; ++q) {
            const int d = hb == 3 ? q + 1 : hb - q;    // use order of the reference
            b[q] = d <= avail
                ? p.upper_l[static_cast<std::size_t>(d - 1) * w + static_cast<std::size_t>(j)] : 0.0F;
        }
    }
    out.eligible = delayed;
    if (delayed && out.ring_ok_transposed) {
        const auto fs = static_cast<std::size_t>(out.forward_stride);
        auto start_of = [&](std::size_t j) {
            int v;
            std::memcpy(&v, &out.forward[j * fs], sizeof(int));
            return v;
        };
        int span = 0;
        for (std::size_t g = 0; g < padded; g += 4) span = std::max(span, start_of(g + 3) + window - start_of(g));
        const int u = span <= 12 ? 12 : span <= 16 ? 16 : 0;
        if (u) {
            out.group_union = u;
            out.group_stride = 8 + 4 * u + round4(4 * hb);
            const auto gs = static_cast<std::size_t>(out.group_stride);
            out.forward_groups.assign(padded / 4 * gs, 0.0F);
            for (std::size_t g = 0; g < padded; g += 4) {
                float *d = out.forward_groups.data() + g / 4 * gs;
                const int base = start_of(g);
                const int ring_offset = (base & (kStreamRing - 1)) * kTRingPitch;
                const int need = start_of(g + 3) + window;
                std::memcpy(&d[0], &base, sizeof(int));
                std::memcpy(&d[1], &ring_offset, sizeof(int));
                std::memcpy(&d[2], &need, sizeof(int));
                for (std::size_t q = 0; q < 4; ++q) {
                    const float *r = out.forward.data() + (g + q) * fs;
                    d[4 + q] = r[1];
                    const int at = start_of(g + q) - base;
                    for (int k = 0; k < window; ++k) d[8 + q * u + static_cast<std::size_t>(at + k)] = r[4 + k];
                    for (int i = 0; i < hb; ++i)
                        d[8 + 4 * static_cast<std::size_t>(u) + q * static_cast<std::size_t>(hb) + i] = r[4 + window + i];
                }
            }
            const auto bs = static_cast<std::size_t>(out.backward_stride);
            const auto bg = static_cast<std::size_t>(round4(4 * hb));
            out.backward_groups.assign(padded / 4 * bg, 0.0F);
            for (std::size_t j = 0; j < padded; ++j)
                for (int i = 0; i < hb; ++i)
                    out.backward_groups[j / 4 * bg + (j % 4) * static_cast<std::size_t>(hb) + static_cast<std::size_t>(i)]
                        = out.backward[j * bs + static_cast<std::size_t>(i)];
        }
    }
    out.segmentable = delayed && out.ring_ok_transposed && fworst <= std::ldexp(1.0, -26);
    if (out.exact) {
        const auto fs = static_cast<std::size_t>(out.forward_stride), bs = static_cast<std::size_t>(out.backward_stride);
        auto transfer = [&](int margin) {
            const int span = margin * chunk;
            double t = 0.0;
            std::vector<double> z(static_cast<std::size_t>(span + hb));
            for (int k = 1; k < chunks; ++k) {
                const int a = k * chunk;
                if (a + span > n) break;
                for (int e = 0; e < hb; ++e) {
                    std::fill(z.begin(), z.end(), 0.0);
                    z[static_cast<std::size_t>(hb - 1 - e)] = 1.0;           // z[i]: position a - hb + i
                    for (int i = a; i < a + span; ++i) {
                        const float *f = out.forward.data() + static_cast<std::size_t>(i) * fs;
                        double s = 0.0;
                        for (int q = 0; q < hb; ++q)
                            s += static_cast<double>(f[4 + window + q]) * z[static_cast<std::size_t>(i - (hb - q) - a + hb)];
                        z[static_cast<std::size_t>(i - a + hb)] = s * static_cast<double>(f[1]);
                    }
                    for (int q = 0; q < hb; ++q) t = std::max(t, std::abs(z[static_cast<std::size_t>(span + q)]));
                    std::fill(z.begin(), z.end(), 0.0);
                    z[static_cast<std::size_t>(span + e)] = 1.0;             // z[i]: position a + i
                    for (int i = a + span - 1; i >= a; --i) {
                        const float *b = out.backward.data() + static_cast<std::size_t>(i) * bs;
                        double s = 0.0;
                        for (int q = 0; q < hb; ++q) {
                            const int d = hb == 3 ? q + 1 : hb - q;
                            s += static_cast<double>(b[q]) * z[static_cast<std::size_t>(i + d - a)];
                        }
                        z[static_cast<std::size_t>(i - a)] = -s;
                    }
                    for (int q = 0; q < hb; ++q) t = std::max(t, std::abs(z[static_cast<std::size_t>(q)]));
                }
            }
            return t;
        };
        for (int margin = 1; margin <= 4; ++margin) {
            out.exact_margin_transfer = transfer(margin);
            if (chunks >= 2 * margin + 1 && out.exact_margin_transfer <= std::ldexp(1.0, -26)) {
                out.exact_margin = margin;
                break;
            }
        }
    }
    out.chunk_first_block.resize(static_cast<std::size_t>(chunks));
    for (int k = 0; k < chunks; ++k) out.chunk_first_block[static_cast<std::size_t>(k)] = s0[static_cast<std::size_t>(k) * chunk] / 16 * 16;

    if (delayed && out.ring_ok_transposed && window <= 16) {
        const int pl = round4(2 * hb);
        out.paired = true;
        out.paired_forward_stride = 4 + 2 * window + pl;
        out.paired_backward_stride = std::max(4, pl);
        out.paired_forward.assign(padded * static_cast<std::size_t>(out.paired_forward_stride), 0.0F);
        out.paired_backward.assign(padded * static_cast<std::size_t>(out.paired_backward_stride), 0.0F);
        for (std::size_t j = 0; j < padded; ++j) {
            const float *f = out.forward.data() + j * static_cast<std::size_t>(out.forward_stride);
            float *g = out.paired_forward.data() + j * static_cast<std::size_t>(out.paired_forward_stride);
            g[0] = f[0];                                   // window start bits
            g[1] = f[1];                                   // inverse diagonal, twice
            g[2] = f[1];
            int start = 0;                                 // ring offset in float2 units
            std::memcpy(&start, &f[0], sizeof(int));
            const int ring_offset = (start & (kStreamRing - 1)) * (kPairedRingPitch / 2);
            std::memcpy(&g[3], &ring_offset, sizeof(int));
            for (int k = 0; k < window + hb; ++k) {        // weights, then -lower
                g[4 + 2 * k] = f[4 + k];
                g[4 + 2 * k + 1] = f[4 + k];
            }
            const float *b = out.backward.data() + j * static_cast<std::size_t>(out.backward_stride);
            float *h = out.paired_backward.data() + j * static_cast<std::size_t>(out.paired_backward_stride);
            for (int q = 0; q < hb; ++q) {
                h[2 * q] = -b[q];
                h[2 * q + 1] = -b[q];
            }
        }
    }
    return out;
}

StreamPack64 pack_stream_plan64(const AxisPlan &p, int chunk, int ring, bool hb_supported) {
    StreamPack64 out;
    const int n = p.destination_size, m = p.source_size, hb = p.half_bandwidth;
    if (!hb_supported || !p.requires_float64()) return out;
    int span = 1;
    for (int j = 0; j < n; ++j) {
        const auto b = p.transpose_offsets[j], e = p.transpose_offsets[j + 1];
        if (b < e) span = std::max(span, p.transpose_indices[e - 1] - p.transpose_indices[b] + 1);
    }
    const int window = round4(span);
    if (window > 16 || window > m) return out;
    std::vector<int> s0(static_cast<std::size_t>(n));
    int previous = 0;
    for (int j = 0; j < n; ++j) {
        const auto b = p.transpose_offsets[j], e = p.transpose_offsets[j + 1];
        int first = b < e ? p.transpose_indices[b] : previous;
        first = std::min(first, m - window);
        if (first < previous) return out;
        s0[static_cast<std::size_t>(j)] = first;
        previous = first;
    }
    if (!ring_fits(s0, window, m, 16, ring)) return out;
    const int fs = (3 + window + hb + 1) / 2 * 2;          // doubles, even
    const int bs = std::max(2, (hb + 1) / 2 * 2);
    const auto padded = static_cast<std::size_t>((n + chunk - 1) / chunk) * static_cast<std::size_t>(chunk);
    out.forward.assign(padded * static_cast<std::size_t>(fs), 0.0);
    out.backward.assign(padded * static_cast<std::size_t>(bs), 0.0);
    const auto w = static_cast<std::size_t>(n);
    for (std::size_t j = 0; j < padded; ++j) {
        double *f = out.forward.data() + j * static_cast<std::size_t>(fs);
        const bool real = j < w;
        const int start = real ? s0[j] : s0.back();
        int count = 0;
        if (real) {
            for (auto k = p.transpose_offsets[j]; k < p.transpose_offsets[j + 1]; ++k) {
                const int at = p.transpose_indices[k] - start;
                f[3 + at] = p.transpose_weights_f64[k];
                count = std::max(count, at + 1);
            }
            f[1] = p.ldlt_bands_f64[j] + DBL_EPSILON;      // band 0 holds D
            f[2] = 1.0 / f[1];
            for (int q = 0; q < hb; ++q) {
                const int d = hb - q;                          // d = hb..1
                if (static_cast<std::size_t>(d) <= j)
                    f[3 + window + q] = p.ldlt_bands_f64[static_cast<std::size_t>(d) * w + j - static_cast<std::size_t>(d)];
            }
            double *b = out.backward.data() + j * static_cast<std::size_t>(bs);
            const auto avail = std::min<std::size_t>(static_cast<std::size_t>(hb), w - j - 1);
            for (int q = 0; q < hb; ++q) {
                const int d = hb - q;
                if (static_cast<std::size_t>(d) <= avail)
                    b[q] = p.ldlt_bands_f64[static_cast<std::size_t>(d) * w + j];
            }
        } else {
            f[1] = 1.0;
            f[2] = 1.0;
        }
        const long long head = static_cast<long long>(static_cast<std::uint32_t>(start))
            | (static_cast<long long>(count) << 32);
        std::memcpy(&f[0], &head, sizeof(head));
    }
    out.eligible = true;
    out.window = window;
    out.forward_stride = 2 * fs;
    out.backward_stride = 2 * bs;

    // Segment margins: a unit in any history slot entering position a (the
    // forward recurrence of the undivided values, z_i = -sum_d L z_{i-d}) or
    // any carry slot entering position a from above (x_i = -sum_d L x_{i+d}),
    // pushed through `margin` chunks; the smallest margin of 2..4 chunks that
    // leaves less than 2^-60 of it.
    const int chunks = static_cast<int>(padded) / chunk;
    auto transfer = [&](int margin) {
        const int span64 = margin * chunk;
        double worst = 0.0;
        std::vector<double> z(static_cast<std::size_t>(span64 + hb));
        for (int k = 1; k < chunks; ++k) {
            const int a = k * chunk;
            for (int e = 0; e < hb; ++e) {
                std::fill(z.begin(), z.end(), 0.0);
                z[static_cast<std::size_t>(hb - 1 - e)] = 1.0;          // z[i] holds position a - hb + i
                const int hi = std::min(n, a + span64);
                for (int i = a; i < hi; ++i) {
                    const double *f = out.forward.data() + static_cast<std::size_t>(i) * static_cast<std::size_t>(fs);
                    double s = 0.0;
                    for (int q = 0; q < hb; ++q) s += f[3 + window + q] * z[static_cast<std::size_t>(i - (hb - q) - a + hb)];
                    z[static_cast<std::size_t>(i - a + hb)] = -s;
                }
                if (hi == a + span64)
                    for (int q = 0; q < hb; ++q) worst = std::max(worst, std::abs(z[static_cast<std::size_t>(span64 + q)]));
            }
            const int top = a + span64;                                   // carry enters below `top`
            if (top > n) continue;
            for (int e = 0; e < hb; ++e) {
                std::fill(z.begin(), z.end(), 0.0);
                z[static_cast<std::size_t>(span64 + e)] = 1.0;           // z[i] holds position a + i
                for (int i = top - 1; i >= a; --i) {
                    const double *b = out.backward.data() + static_cast<std::size_t>(i) * static_cast<std::size_t>(bs);
                    double s = 0.0;
                    for (int q = 0; q < hb; ++q) s += b[q] * z[static_cast<std::size_t>(i + (hb - q) - a)];
                    z[static_cast<std::size_t>(i - a)] = -s;
                }
                for (int q = 0; q < hb; ++q) worst = std::max(worst, std::abs(z[static_cast<std::size_t>(q)]));
            }
        }
        return worst;
    };
    for (int margin = 2; margin <= 4; ++margin) {
        out.margin_transfer = transfer(margin);
        if (chunks >= 2 * margin && out.margin_transfer <= std::ldexp(1.0, -60)) {
            out.margin = margin;
            break;
        }
    }
    out.segmentable = out.margin > 0;
    out.chunk_first_block.resize(static_cast<std::size_t>(chunks));
    for (int k = 0; k < chunks; ++k)
        out.chunk_first_block[static_cast<std::size_t>(k)] = s0[std::min<std::size_t>(static_cast<std::size_t>(k) * chunk, w - 1)] / 16 * 16;
    return out;
}

} // namespace dsmvc_gb
