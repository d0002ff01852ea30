// Two-pass transposing kernels of the Float64 route (plans that retain
// Float64 on both axes).
//
// The warp layout of the Float32 transposing kernels (a warp owns 32 vectors,
// one per lane; source blocks of 16 samples fetched by the whole warp with
// coalesced 16-byte loads into a shared ring, here of doubles; records staged
// per chunk of 32 destinations through cp.async), with the arithmetic of the
// CPU scalar Float64 route (solve_banded_ldlt, src/axis_plan.cpp:793-823 and
// detail::inverse_axis_f64, :1193-1257): every multiply and add rounded on
// its own (__dmul_rn, __dadd_rn, __dsub_rn, __ddiv_rn), the gather over the
// A^T entries in CSR order, the unit-L forward substitution on the undivided
// values, the division by D + DBL_EPSILON, the backward substitution term by
// term.  Two sweeps: the forward values go to a Float64 plane laid out like
// the output (the intermediate itself in the first pass), the backward sweep
// reads them back.  Results equal the CPU's bit for bit.
//
// FUSED variant (the default route): the same sweeps with every multiply-add
// fused (fma, one rounding instead of two) and the division by D + DBL_EPSILON
// replaced by a product with its reciprocal (rounded once on the host): less
// than half the FP64 pipe operations of the CPU order.  The Float64 results
// differ from the CPU's by a few double ULPs, far below a float32 ULP, so
// outputs stay within the <= 1 float32 ULP / <= 1 code contract.
#pragma once

#include "tstream_impl.cuh"

#include <cfloat>

namespace dsmvc_gb {
namespace {

constexpr int kXPitch = 34;                          // doubles between ring rows
constexpr int kXRows = kTRing + kTDup;               // 32 rows + the first 16 again
constexpr int kXRingDoubles = kXRows * kXPitch;

template <class T> __device__ __forceinline__ double xload(T v, const Conversion &c) {
    return __dmul_rn(__dsub_rn(static_cast<double>(v), static_cast<double>(c.in_offset)),
                     static_cast<double>(c.in_scale));
}
template <> __device__ __forceinline__ double xload<float>(float v, const Conversion &) { return v; }
template <> __device__ __forceinline__ double xload<double>(double v, const Conversion &) { return v; }
template <class T> __device__ __forceinline__ bool xfinite(T) { return true; }
template <> __device__ __forceinline__ bool xfinite<float>(float v) { return isfinite(v); }

// src/cpu_executor.cpp:1617-1645 for integer outputs; Float32 rounds to
// nearest; the Float64 intermediate keeps the value.
template <class T> __device__ __forceinline__ T xstore(double v, const Conversion &c, std::uint32_t &flags) {
    const double s = __dadd_rn(__dmul_rn(v, static_cast<double>(c.out_scale)), static_cast<double>(c.out_offset));
    if (!isfinite(v) || !isfinite(s)) {
        flags |= dev::kStatusNonFiniteOutput;
        return T{};
    }
    return static_cast<T>(__double2uint_rn(fmin(fmax(s, 0.0), static_cast<double>(c.out_max))));
}
template <> __device__ __forceinline__ float xstore<float>(double v, const Conversion &, std::uint32_t &flags) {
    const float f = __double2float_rn(v);
    if (!isfinite(v) || !isfinite(f)) flags |= dev::kStatusNonFiniteOutput;
    return f;
}
template <> __device__ __forceinline__ double xstore<double>(double v, const Conversion &, std::uint32_t &) {
    return v;
}

// Ring feeder of one warp for the Float64 kernels: blocks of 16 samples of
// the warp's 32 vectors, converted to double.
template <class In>
struct WarpFeeder64 {
    static constexpr int SPL = 16 / static_cast<int>(sizeof(In));   // samples per lane load
    static constexpr int LPV = kTBlock / SPL;                       // lanes per vector
    static constexpr int VPI = 32 / LPV;                            // vectors per load
    static constexpr int NI = 32 / VPI;                             // loads per block
    const In *base;
    std::int64_t stride;
    int size, have, vectors, lane;
    bool vec_ok;
    double *ring;            // ring[row * kXPitch + vector]
    Conversion conv;
    std::uint32_t flags = 0;
    uint4 pend[NI];
    bool pend_ok;

    __device__ __forceinline__ void put(int s, int v, In raw) {
        if (!xfinite(raw)) flags |= dev::kStatusNonFiniteInput;
        const double x = xload(raw, conv);
        const int row = s & (kTRing - 1);
        double *r = ring + row * kXPitch + v;
        r[0] = x;
        if (row < kTDup) r[kTRing * kXPitch] = x;
    }

    __device__ __forceinline__ void issue() {
        pend_ok = vec_ok && have + kTBlock <= size;
        if (!pend_ok) return;
#pragma unroll
        for (int i = 0; i < NI; ++i) {
            int v = i * VPI + lane / LPV;
            v = v < vectors ? v : vectors - 1;
            pend[i] = __ldg(reinterpret_cast<const uint4 *>(base + v * stride + have + (lane % LPV) * SPL));
        }
    }

    // `first`: a multiple of 16 at most the first window start.
    __device__ __forceinline__ void start(int first = 0) {
        have = first;
        issue();
    }

    __device__ __forceinline__ void ensure(int need) {
        if (have >= need) return;
        while (have < need) {
            if (pend_ok) {
#pragma unroll
                for (int i = 0; i < NI; ++i) {
                    const int v = i * VPI + lane / LPV;
                    const In *vals = reinterpret_cast<const In *>(&pend[i]);
#pragma unroll
                    for (int k = 0; k < SPL; ++k) put(have + (lane % LPV) * SPL + k, v, vals[k]);
                }
                have += kTBlock;
                issue();
            } else {
                const int v = lane < vectors ? lane : vectors - 1;
                put(have, lane, __ldg(base + v * stride + have));
                have += 1;
            }
        }
        __syncwarp();
    }
};

// Record words (doubles): forward [s0 | count << 32 (bits), D + DBL_EPSILON,
// 1 / (D + DBL_EPSILON), window weights, L factors for d = HB..1, padding to
// even]; backward [L factors of the following destinations for d = HB..1,
// padding to even].
template <int HB, bool FUSED, class In, class Out>
__global__ void __launch_bounds__(kTMaxThreads)
tsolve64_kernel(const StreamJob *__restrict__ jobs, int job_count, int record_floats, std::uint32_t *status) {
    constexpr int LC = kTChunk;
    extern __shared__ __align__(16) float smem[];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nthreads = static_cast<int>(blockDim.x);
    const int cta_warp = static_cast<int>(blockIdx.x) * (nthreads >> 5);
    const StreamJob &job = jobs[find_tjob(jobs, job_count, cta_warp + warp)];
    const StreamJob &lead = jobs[find_tjob(jobs, job_count, cta_warp)];
    const dev::StreamPlanView p = lead.plan;
    const int n = p.destination_size;
    const int chunks = (n + kTChunk - 1) / kTChunk;
    // Chunks stored: [ca, cb); a segment (chunk_end > 0) sweeps forward over
    // [fc0, fce] from a zero history and backward from a zero carry after
    // fce, `margin` chunks beyond its range on either side (within the
    // vector), with its forward values in its own region starting at chunk
    // fc0.  Every warp of a CTA serves the same plan and range.
    const bool segment = lead.chunk_end > 0;
    const int ca = lead.chunk_begin;
    const int cb = segment ? lead.chunk_end : chunks;
    const int fc0 = segment ? max(ca - lead.margin, 0) : 0;
    const int fce = segment ? min(cb + lead.margin, chunks) - 1 : chunks - 1;
    const int ybase = fc0 * kTChunk;
    const int per_buffer = kTChunk * record_floats;
    float *bufs = smem;
    double *ring = reinterpret_cast<double *>(smem + 3 * per_buffer) + warp * kXRingDoubles;

    int warp_first = (cta_warp + warp - job.first_block) * 32;
    int warp_vectors = job.vectors - warp_first;
    const bool idle = warp_vectors <= 0;
    if (warp_vectors <= 0) {
        warp_first = job.vectors - 1;
        warp_vectors = 1;
    } else if (warp_vectors > 32) {
        warp_vectors = 32;
    }
    const bool active = (cta_warp + warp - job.first_block) * 32 + lane < job.vectors;
    const int v = warp_first + (lane < warp_vectors ? lane : 0);

    WarpFeeder64<In> feed;
    feed.base = static_cast<const In *>(job.in) + warp_first * job.in_vec;
    feed.stride = job.in_vec;
    feed.size = p.source_size;
    feed.vectors = warp_vectors;
    feed.lane = lane;
    feed.ring = ring;
    feed.conv = job.conv;
    feed.vec_ok = (reinterpret_cast<std::uintptr_t>(job.in) % 16 == 0)
        && (job.in_vec * static_cast<std::int64_t>(sizeof(In))) % 16 == 0;
    if (!idle) feed.start(fc0 > 0 ? lead.first_sample : 0);

    double *yplane = reinterpret_cast<double *>(job.y) + v;
    Out *out = static_cast<Out *>(job.out) + v;
    const int fs = p.forward_stride / 2, bs = p.backward_stride / 2;   // doubles
    const int kw = p.window;
    std::uint32_t flags = 0;

    // ---- forward sweep ---------------------------------------------------
    tstage(bufs + (fc0 % 3) * per_buffer, p, fc0, tid, nthreads);
    tcp_commit();
    if (fc0 + 1 <= fce) tstage(bufs + ((fc0 + 1) % 3) * per_buffer, p, fc0 + 1, tid, nthreads);
    tcp_commit();
    double z[HB];                                        // undivided forward values, newest first
#pragma unroll
    for (int d = 0; d < HB; ++d) z[d] = 0.0;
    for (int c = fc0; c <= fce; ++c) {
        tcp_wait_one();
        __syncthreads();
        const double *fwd = reinterpret_cast<const double *>(bufs + (c % 3) * per_buffer);
        const int j0 = c * LC;
        if (!idle) {
#pragma unroll 1
            for (int t = 0; t < LC; ++t) {
                const int j = j0 + t;
                if (j >= n) break;
                const double *rec = fwd + t * fs;
                const long long head = __double_as_longlong(rec[0]);
                const int s0 = static_cast<int>(head & 0xffffffffLL), count = static_cast<int>(head >> 32);
                feed.ensure(min(s0 + kw, p.source_size));
                const double *win = ring + (s0 & (kTRing - 1)) * kXPitch + lane;
                double sum = 0.0;
                if constexpr (FUSED) {
                    for (int k = 0; k < count; ++k) sum = fma(rec[3 + k], win[k * kXPitch], sum);
#pragma unroll
                    for (int q = 0; q < HB; ++q) sum = fma(-rec[3 + kw + q], z[HB - q - 1], sum);
                } else {
                    for (int k = 0; k < count; ++k) sum = __dadd_rn(sum, __dmul_rn(rec[3 + k], win[k * kXPitch]));
#pragma unroll
                    for (int q = 0; q < HB; ++q) {             // d = HB - q, descending
                        const int d = HB - q;
                        sum = __dsub_rn(sum, __dmul_rn(rec[3 + kw + q], z[d - 1]));
                    }
                }
#pragma unroll
                for (int d = HB - 1; d > 0; --d) z[d] = z[d - 1];
                z[0] = sum;
                if (active)
                    yplane[static_cast<std::int64_t>(j - ybase) * job.y_elem] =
                        FUSED ? sum * rec[2] : __ddiv_rn(sum, rec[1]);
            }
        }
        __syncthreads();
        if (c + 2 <= fce) tstage(bufs + ((c + 2) % 3) * per_buffer, p, c + 2, tid, nthreads);
        tcp_commit();
    }
    flags |= feed.flags;

    // ---- backward sweep --------------------------------------------------
    asm volatile("cp.async.wait_all;\n" ::: "memory");
    __syncthreads();
    tstage(bufs, p, fce, tid, nthreads);
    tcp_commit();
    if (fce - 1 >= ca) tstage(bufs + per_buffer, p, fce - 1, tid, nthreads);
    tcp_commit();
    double x[HB];                                        // following results, nearest first
#pragma unroll
    for (int d = 0; d < HB; ++d) x[d] = 0.0;
    for (int c = fce, k = 0; c >= ca; --c, ++k) {
        tcp_wait_one();
        __syncthreads();
        const double *bwd = reinterpret_cast<const double *>(bufs + (k % 3) * per_buffer) + kTChunk * fs;
        const int j0 = c * LC;
        if (!idle && active) {
            const int top = min(LC, n - j0) - 1;
            double y_next = yplane[static_cast<std::int64_t>(j0 + top - ybase) * job.y_elem];
            const bool store = c < cb;
#pragma unroll 1
            for (int t = top; t >= 0; --t) {
                const double yt = y_next;
                if (t > 0) y_next = yplane[static_cast<std::int64_t>(j0 + t - 1 - ybase) * job.y_elem];
                const double *rec = bwd + t * bs;
                double xt = yt;
#pragma unroll
                for (int q = 0; q < HB; ++q) {                 // d = HB - q, descending
                    const int d = HB - q;
                    xt = FUSED ? fma(-rec[q], x[d - 1], xt) : __dsub_rn(xt, __dmul_rn(rec[q], x[d - 1]));
                }
#pragma unroll
                for (int d = HB - 1; d > 0; --d) x[d] = x[d - 1];
                x[0] = xt;
                if (store) out[static_cast<std::int64_t>(j0 + t) * job.out_elem] = xstore<Out>(xt, job.conv, flags);
            }
        }
        __syncthreads();
        if (c - 2 >= ca) tstage(bufs + ((k + 2) % 3) * per_buffer, p, c - 2, tid, nthreads);
        tcp_commit();
    }
    if (flags && active) atomicOr(status, flags);
}

template <int HB, bool FUSED, class In, class Out>
int x64launch_typed(const StreamJob *jobs, int count, int blocks, int threads, int record_floats,
                    std::uint32_t *status, cudaStream_t s) {
    if (threads < 32 || threads > kTMaxThreads || threads % 32) return static_cast<int>(cudaErrorInvalidValue);
    const int smem = 3 * kTChunk * record_floats * static_cast<int>(sizeof(float))
        + threads / 32 * kXRingDoubles * static_cast<int>(sizeof(double));
    auto kernel = tsolve64_kernel<HB, FUSED, In, Out>;
    static SmemLimit limit;
    if (const cudaError_t e = limit.ensure(kernel, smem); e != cudaSuccess) return static_cast<int>(e);
    kernel<<<blocks, threads, smem, s>>>(jobs, count, record_floats, status);
    return static_cast<int>(cudaGetLastError());
}

template <int HB, bool FUSED>
int x64launch_fused(const StreamJob *jobs, int count, int blocks, int threads, dev::Sample in, dev::Sample out,
                    int record_floats, std::uint32_t *status, cudaStream_t s) {
    using dev::Sample;
    if (out == Sample::f64) {
        if (in == Sample::f32) return x64launch_typed<HB, FUSED, float, double>(jobs, count, blocks, threads, record_floats, status, s);
        if (in == Sample::u16) return x64launch_typed<HB, FUSED, std::uint16_t, double>(jobs, count, blocks, threads, record_floats, status, s);
        if (in == Sample::u8) return x64launch_typed<HB, FUSED, std::uint8_t, double>(jobs, count, blocks, threads, record_floats, status, s);
    }
    if (in == Sample::f64) {
        if (out == Sample::f64) return x64launch_typed<HB, FUSED, double, double>(jobs, count, blocks, threads, record_floats, status, s);
        if (out == Sample::f32) return x64launch_typed<HB, FUSED, double, float>(jobs, count, blocks, threads, record_floats, status, s);
        if (out == Sample::u16) return x64launch_typed<HB, FUSED, double, std::uint16_t>(jobs, count, blocks, threads, record_floats, status, s);
        if (out == Sample::u8) return x64launch_typed<HB, FUSED, double, std::uint8_t>(jobs, count, blocks, threads, record_floats, status, s);
    }
    return static_cast<int>(cudaErrorInvalidValue);
}

template <int HB>
int x64launch_hb(const StreamJob *jobs, int count, int blocks, int threads, dev::Sample in, dev::Sample out,
                 int record_floats, bool fused, std::uint32_t *status, cudaStream_t s) {
    return fused ? x64launch_fused<HB, true>(jobs, count, blocks, threads, in, out, record_floats, status, s)
                 : x64launch_fused<HB, false>(jobs, count, blocks, threads, in, out, record_floats, status, s);
}

} // namespace
} // namespace dsmvc_gb
