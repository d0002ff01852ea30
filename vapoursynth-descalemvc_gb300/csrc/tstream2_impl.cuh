// Paired transposing streaming kernels: the two passes of a Float32 2D
// descale with two vectors per lane.
//
// Same algorithm and data flow as tstream_impl.cuh (exact forward
// substitution, chunk-delayed backward substitution from a zero carry one
// chunk ahead, a shared sample ring fed by warp-wide 16-byte loads, chunk
// records staged through cp.async), but a warp owns 64 vectors and lane l
// owns the adjacent vectors 2l and 2l+1, so every arithmetic instruction is a
// packed float2 one (fma.rn.f32x2 and friends) serving two outputs:
//
//  * records hold every coefficient twice ([w0, w0, w1, w1, ...]), so one
//    16-byte record load yields two coefficient pairs; backward factors are
//    stored negated, so x = y + sum(-u * x) (exactly y - sum(u * x));
//  * the ring is [sample row][64 vectors] floats, so a lane's two window
//    samples are one 8-byte load; rows are 66 floats apart (conflict-free
//    scatter for every load pattern) and the first 16 rows are stored again
//    after the 32 resident rows, so any window of up to 16 samples is
//    contiguous;
//  * the previous chunk's forward values wait in shared memory (one 8-byte
//    store and load per destination and lane) instead of registers.
//
// Admitted per plan by the host (window <= 16, the grouped ring replay of
// the unpaired kernels, the backward decay check).  Per output, the
// operations and their order are those of the unpaired kernels, each half of
// a packed operation rounding like its scalar form, so both kernels give
// identical results.
#pragma once

#include "kernels.cuh"
#include "smem_limit.cuh"
#include "stream.cuh"

#include <cuda_runtime.h>

#include <cstdint>

namespace dsmvc_gb {
namespace {

using dev::Conversion;
using dev::StreamJob;

constexpr int kPResident = 32;                 // samples resident in a ring
constexpr int kPRows = 48;                     // 32 rows + the first 16 again
constexpr int kPPitch = kPairedRingPitch;      // floats between ring rows
constexpr int kPRingFloats = kPRows * kPPitch;
constexpr int kPChunk = kStreamChunk;
constexpr int kPYFloats = kPChunk * 64;        // previous chunk, per warp
constexpr int kPMaxThreads = 256;
constexpr int kPBlock = 16;                    // samples per warp load block

__device__ __forceinline__ int find_pjob(const StreamJob *jobs, int count, int block) {
    int lo = 0, hi = count - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (jobs[mid].first_block <= block) lo = mid; else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ void pcp_async16(float *smem, const float *gmem) {
    const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" :: "r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void pcp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void pcp_wait_one() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }

template <class T> __device__ __forceinline__ float pin(T v, const Conversion &c) {
    return (static_cast<float>(v) - c.in_offset) * c.in_scale;
}
template <> __device__ __forceinline__ float pin<float>(float v, const Conversion &) { return v; }

template <class T> __device__ __forceinline__ T pout(float v, const Conversion &c) {
    float s = __fadd_rn(__fmul_rn(v, c.out_scale), c.out_offset);
    s = fminf(fmaxf(s, 0.0f), static_cast<float>(c.out_max));
    return static_cast<T>(__float2uint_rn(s));
}
template <> __device__ __forceinline__ float pout<float>(float v, const Conversion &) { return v; }

__device__ __forceinline__ float4 plds4(const float *p) { return *reinterpret_cast<const float4 *>(p); }
__device__ __forceinline__ float2 lo2(const float4 &v) { return make_float2(v.x, v.y); }
__device__ __forceinline__ float2 hi2(const float4 &v) { return make_float2(v.z, v.w); }

// Paired record strides (floats); compile-time with a compile-time window.
template <int HB, int K> __device__ __forceinline__ int pfwd_stride(const dev::StreamPlanView &p) {
    return K > 0 ? 4 + 2 * K + (2 * HB + 3) / 4 * 4 : p.forward_stride;
}
template <int HB, int K> __device__ __forceinline__ int pbwd_stride(const dev::StreamPlanView &p) {
    return K > 0 ? (2 * HB + 3) / 4 * 4 : p.backward_stride;
}

// Cooperative ring feeder of one warp and its 64 vectors.  Block b covers
// samples [16 b, 16 b + 16).
template <class In>
struct PairFeeder {
    static constexpr int SPL = 16 / static_cast<int>(sizeof(In));   // samples per lane load
    static constexpr int LPV = kPBlock / SPL;                       // lanes per vector
    static constexpr int VPI = 32 / LPV;                            // vectors per load
    static constexpr int NI = 64 / VPI;                             // loads per block
    const In *base;          // vector 0 of the warp
    std::int64_t stride;     // samples between vectors
    int size;                // samples per vector
    int have;                // samples in the ring
    int vectors;             // valid vectors of the warp (1..64)
    bool vec_ok;             // 16-byte aligned vectors
    int lane;
    float *ring;             // ring[row * kPPitch + vector]
    Conversion conv;
    uint4 pend[NI];
    bool pend_ok;

    __device__ __forceinline__ void put(int s, int v, float x) {
        const int row = s & (kPResident - 1);
        float *r = ring + row * kPPitch + v;
        r[0] = x;
        if (row < kPRows - kPResident) r[kPResident * kPPitch] = x;
    }

    __device__ __forceinline__ void issue() {
        pend_ok = vec_ok && have + kPBlock <= size;
        if (!pend_ok) return;
#pragma unroll
        for (int i = 0; i < NI; ++i) {
            int v = i * VPI + lane / LPV;
            v = v < vectors ? v : vectors - 1;
            const In *p = base + v * stride + have + (lane % LPV) * SPL;
            pend[i] = __ldg(reinterpret_cast<const uint4 *>(p));
        }
    }

    __device__ __forceinline__ void start() {
        have = 0;
        issue();
    }

    // Makes samples [0, need) resident (need <= size) and visible warp-wide.
    __device__ __forceinline__ void ensure(int need) {
        if (have >= need) return;
        while (have < need) {
            if (pend_ok) {
                // A block starts on a multiple of 16: all of it is in the
                // duplicated rows or none of it is.
                const bool dup = (have & (kPResident - 1)) < kPRows - kPResident;
#pragma unroll
                for (int i = 0; i < NI; ++i) {
                    const int v = i * VPI + lane / LPV;
                    const In *vals = reinterpret_cast<const In *>(&pend[i]);
                    const int s = have + (lane % LPV) * SPL;
                    float *r = ring + (s & (kPResident - 1)) * kPPitch + v;
#pragma unroll
                    for (int k = 0; k < SPL; ++k) {
                        const float x = pin(vals[k], conv);
                        r[k * kPPitch] = x;
                        if (dup) r[(kPResident + k) * kPPitch] = x;
                    }
                }
                have += kPBlock;
                issue();
            } else {
                // Unaligned vectors or the tail: one sample of each of the
                // lane's two vectors.
                const int v0 = 2 * lane < vectors ? 2 * lane : vectors - 1;
                const int v1 = 2 * lane + 1 < vectors ? 2 * lane + 1 : vectors - 1;
                put(have, 2 * lane, pin(__ldg(base + v0 * stride + have), conv));
                put(have, 2 * lane + 1, pin(__ldg(base + v1 * stride + have), conv));
                have += 1;
            }
        }
        __syncwarp();
    }
};

__device__ __forceinline__ void pstage(float *buf, const dev::StreamPlanView &p, int chunk, int tid, int nthreads) {
    const int fs = p.forward_stride, bs = p.backward_stride;
    const float *gf = p.forward + static_cast<std::int64_t>(chunk) * kPChunk * fs;
    const float *gb = p.backward + static_cast<std::int64_t>(chunk) * kPChunk * bs;
    for (int i = tid * 4; i < kPChunk * fs; i += nthreads * 4) pcp_async16(buf + i, gf + i);
    float *bb = buf + kPChunk * fs;
    for (int i = tid * 4; i < kPChunk * bs; i += nthreads * 4) pcp_async16(bb + i, gb + i);
}

// Forward substitution of chunk destinations [j0, j0 + 32) into y[t];
// hist[HB + k] (k = -HB..-1) holds the previous chunk's last HB values.
template <int HB, int K, class Feed>
__device__ __forceinline__ void pforward(float2 (&y)[kPChunk], const float2 (&hist)[HB > 0 ? HB : 1], int j0,
                                         const dev::StreamPlanView &p, const float *fwd, Feed &feed, int lane) {
    const int fs = pfwd_stride<HB, K>(p);
    const int kw = K > 0 ? K : p.window;
    const int n = p.destination_size;
    const float2 *ring2 = reinterpret_cast<const float2 *>(feed.ring);
#pragma unroll
    for (int t = 0; t < kPChunk; ++t) {
        if (t % 4 == 0) {
            // Window end of the group's last destination (window starts never
            // decrease; padding records repeat the last destination's start).
            const int s_last = __float_as_int(fwd[(t + 3) * fs]);
            const int need = max(s_last, __float_as_int(fwd[t * fs])) + kw;
            feed.ensure(min(need, p.source_size));
        }
        const float *rec = fwd + t * fs;
        const float4 hdr = plds4(rec);
        // Record word 3: the window's ring offset in float2 units.
        const float2 *win = ring2 + lane + __float_as_int(hdr.w);
        // Even and odd taps in two partial sums, as the unpaired kernels.
        float2 se = make_float2(0.0f, 0.0f), so = make_float2(0.0f, 0.0f);
        if constexpr (K > 0) {
#pragma unroll
            for (int k = 0; k < K; k += 2) {
                const float4 w = plds4(rec + 4 + 2 * k);
                se = __ffma2_rn(lo2(w), win[(k + 0) * (kPPitch / 2)], se);
                so = __ffma2_rn(hi2(w), win[(k + 1) * (kPPitch / 2)], so);
            }
        } else {
            for (int k = 0; k < kw; k += 2) {
                const float4 w = plds4(rec + 4 + 2 * k);
                se = __ffma2_rn(lo2(w), win[(k + 0) * (kPPitch / 2)], se);
                so = __ffma2_rn(hi2(w), win[(k + 1) * (kPPitch / 2)], so);
            }
        }
        float2 sum = __fadd2_rn(se, so);
        const float *low = rec + 4 + 2 * kw;
#pragma unroll
        for (int q = 0; q < HB; q += 2) {
            const float4 l = plds4(low + 2 * q);
#pragma unroll
            for (int e = 0; e < 2; ++e) {
                const int qq = q + e;
                if (qq < HB) {
                    const int d = HB - qq;                       // use order d = HB..1
                    const float2 prev = t - d >= 0 ? y[t - d >= 0 ? t - d : 0] : hist[t - d < 0 ? HB + t - d : 0];
                    sum = __ffma2_rn(e == 0 ? lo2(l) : hi2(l), prev, sum);
                }
            }
        }
        y[t] = j0 + t < n ? __fmul2_rn(sum, make_float2(hdr.y, hdr.z)) : make_float2(0.0f, 0.0f);
    }
}

// Zero-carry backward warm-up over the chunk in y; leaves the state
// entering the preceding chunk in `carry`.
template <int HB, int K>
__device__ __forceinline__ void pwarmup(const float2 (&y)[kPChunk], float2 (&carry)[HB > 0 ? HB : 1],
                                        const dev::StreamPlanView &p, const float *bwd) {
    const int bs = pbwd_stride<HB, K>(p);
    float2 w[HB > 0 ? HB : 1];
#pragma unroll
    for (int d = 0; d < HB; ++d) w[d] = make_float2(0.0f, 0.0f);
#pragma unroll
    for (int t = kPChunk - 1; t >= 0; --t) {
        const float *rec = bwd + t * bs;
        float2 sum = make_float2(0.0f, 0.0f);
#pragma unroll
        for (int q = 0; q < HB; q += 2) {
            const float4 u = plds4(rec + 2 * q);
#pragma unroll
            for (int e = 0; e < 2; ++e) {
                const int pos = q + e;
                if (pos < HB) {
                    const int d = HB == 3 ? pos + 1 : HB - pos;
                    const float2 xd = (t + d < kPChunk) ? w[(t + d) % HB] : make_float2(0.0f, 0.0f);
                    sum = __ffma2_rn(e == 0 ? lo2(u) : hi2(u), xd, sum);
                }
            }
        }
        w[t % HB] = __fadd2_rn(y[t], sum);
    }
#pragma unroll
    for (int d = 0; d < HB; ++d) carry[d] = w[d];
}

// Final backward substitution of one chunk from `carry` (x after the
// chunk): y from registers (`ysrc` null) or from the warp's shared copy.
// Stores each x as soon as it is known; leaves the chunk's first HB x
// values in `carry`.
template <int HB, int K, class Out>
__device__ __forceinline__ void pbackward(const float2 (&yreg)[kPChunk], const float2 *ysrc,
                                          float2 (&carry)[HB > 0 ? HB : 1], int j0, const dev::StreamPlanView &p,
                                          const float *bwd, Out *out, std::int64_t out_elem, bool a0, bool a1,
                                          bool pair_store, const Conversion &conv, int lane) {
    const int bs = pbwd_stride<HB, K>(p);
    const int n = p.destination_size;
    float2 w[HB > 0 ? HB : 1];
#pragma unroll
    for (int t = kPChunk - 1; t >= 0; --t) {
        const float *rec = bwd + t * bs;
        const float2 yt = ysrc ? ysrc[t * 32 + lane] : yreg[t];
        float2 sum = make_float2(0.0f, 0.0f);
#pragma unroll
        for (int q = 0; q < HB; q += 2) {
            const float4 u = plds4(rec + 2 * q);
#pragma unroll
            for (int e = 0; e < 2; ++e) {
                const int pos = q + e;
                if (pos < HB) {
                    const int d = HB == 3 ? pos + 1 : HB - pos;
                    const float2 xd = (t + d < kPChunk) ? w[(t + d) % HB] : carry[t + d >= kPChunk ? t + d - kPChunk : 0];
                    sum = __ffma2_rn(e == 0 ? lo2(u) : hi2(u), xd, sum);
                }
            }
        }
        const float2 x = __fadd2_rn(yt, sum);
        w[t % HB] = x;
        if (j0 + t < n) {
            Out *o = out + static_cast<std::int64_t>(j0 + t) * out_elem;
            if (pair_store) {
                *reinterpret_cast<float2 *>(o) = x;
            } else {
                if (a0) o[0] = pout<Out>(x.x, conv);
                if (a1) o[1] = pout<Out>(x.y, conv);
            }
        }
    }
#pragma unroll
    for (int d = 0; d < HB; ++d) carry[d] = w[d];
}

template <int HB, int K, class In, class Out>
__global__ void __launch_bounds__(kPMaxThreads)
tstream2_kernel(const StreamJob *__restrict__ jobs, int job_count, int record_floats) {
    extern __shared__ __align__(16) float smem[];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nthreads = static_cast<int>(blockDim.x), nwarps = nthreads >> 5;
    // Jobs are assigned warps; a CTA's warps share one plan (the host rounds
    // plan changes up to whole CTAs), whose records the CTA copies once.
    const int cta_warp = static_cast<int>(blockIdx.x) * nwarps;
    const StreamJob &job = jobs[find_pjob(jobs, job_count, cta_warp + warp)];
    const dev::StreamPlanView p = jobs[find_pjob(jobs, job_count, cta_warp)].plan;
    const int n = p.destination_size;
    const int per_buffer = kPChunk * record_floats;
    float *bufs = smem;
    float *ring = smem + 3 * per_buffer + warp * kPRingFloats;
    float2 *ysm = reinterpret_cast<float2 *>(smem + 3 * per_buffer + nwarps * kPRingFloats + warp * kPYFloats);

    // The warp's 64 vectors; a warp past its job's last vector only takes
    // part in the CTA's record copies and barriers.
    int warp_first = (cta_warp + warp - job.first_block) * 64;
    int warp_vectors = job.vectors - warp_first;
    const bool idle = warp_vectors <= 0;
    if (warp_vectors <= 0) {
        warp_first = job.vectors - 1;
        warp_vectors = 1;
    } else if (warp_vectors > 64) {
        warp_vectors = 64;
    }
    const int v0 = (cta_warp + warp - job.first_block) * 64 + 2 * lane;
    const bool a0 = v0 < job.vectors, a1 = v0 + 1 < job.vectors;

    PairFeeder<In> feed;
    feed.base = static_cast<const In *>(job.in) + warp_first * job.in_vec;
    feed.stride = job.in_vec;
    feed.size = p.source_size;
    feed.vectors = warp_vectors;
    feed.lane = lane;
    feed.ring = ring;
    feed.conv = job.conv;
    feed.vec_ok = (reinterpret_cast<std::uintptr_t>(job.in) % 16 == 0)
        && (job.in_vec * static_cast<std::int64_t>(sizeof(In))) % 16 == 0;
    if (!idle) feed.start();

    Out *out = static_cast<Out *>(job.out) + (a0 ? v0 : 0);
    const bool pair_store = sizeof(Out) == 4 && a0 && a1 && (job.out_elem % 2 == 0)
        && (reinterpret_cast<std::uintptr_t>(out) % 8 == 0);

    const int chunks = (n + kPChunk - 1) / kPChunk;
    pstage(bufs, p, 0, tid, nthreads);
    pcp_commit();
    if (chunks > 1) pstage(bufs + per_buffer, p, 1, tid, nthreads);
    pcp_commit();

    float2 y[kPChunk];
    float2 hist[HB > 0 ? HB : 1];
    float2 carry[HB > 0 ? HB : 1];
#pragma unroll
    for (int d = 0; d < HB; ++d) hist[d] = make_float2(0.0f, 0.0f);
    for (int c = 0; c < chunks; ++c) {
        pcp_wait_one();
        __syncthreads();
        const float *cur = bufs + (c % 3) * per_buffer;
        const float *prev = bufs + ((c + 2) % 3) * per_buffer;
        const float *cur_b = cur + kPChunk * pfwd_stride<HB, K>(p);
        const float *prev_b = prev + kPChunk * pfwd_stride<HB, K>(p);
        const bool last = c + 1 == chunks;
        if (!idle) {
            pforward<HB, K>(y, hist, c * kPChunk, p, cur, feed, lane);
            if (last) {
#pragma unroll
                for (int d = 0; d < HB; ++d) carry[d] = make_float2(0.0f, 0.0f);
                pbackward<HB, K>(y, nullptr, carry, c * kPChunk, p, cur_b, out, job.out_elem, a0, a1, pair_store,
                                 job.conv, lane);
                if (c > 0)
                    pbackward<HB, K>(y, ysm, carry, (c - 1) * kPChunk, p, prev_b, out, job.out_elem, a0, a1,
                                     pair_store, job.conv, lane);
            } else {
                pwarmup<HB, K>(y, carry, p, cur_b);
                if (c > 0)
                    pbackward<HB, K>(y, ysm, carry, (c - 1) * kPChunk, p, prev_b, out, job.out_elem, a0, a1,
                                     pair_store, job.conv, lane);
#pragma unroll
                for (int t = 0; t < kPChunk; ++t) ysm[t * 32 + lane] = y[t];
#pragma unroll
                for (int d = 0; d < HB; ++d) hist[d] = y[kPChunk - HB + d];
            }
        }
        if (last) break;
        // Every warp is done with chunk c-1's records: fetch chunk c+2.
        __syncthreads();
        if (c + 2 < chunks) pstage(const_cast<float *>(prev), p, c + 2, tid, nthreads);
        pcp_commit();
    }
}

template <int HB, int K, class In, class Out>
int plaunch_typed(const StreamJob *jobs, int count, int blocks, int threads, int record_floats, cudaStream_t s) {
    if (threads < 32 || threads > kPMaxThreads || threads % 32) return static_cast<int>(cudaErrorInvalidValue);
    const int smem = (3 * kPChunk * record_floats + threads / 32 * (kPRingFloats + kPYFloats))
        * static_cast<int>(sizeof(float));
    auto kernel = tstream2_kernel<HB, K, In, Out>;
    static SmemLimit limit;
    if (const cudaError_t e = limit.ensure(kernel, smem); e != cudaSuccess) return static_cast<int>(e);
    kernel<<<blocks, threads, smem, s>>>(jobs, count, record_floats);
    return static_cast<int>(cudaGetLastError());
}

template <int HB, int K>
int plaunch_k(const StreamJob *jobs, int count, int blocks, int threads, dev::Sample in, dev::Sample out,
              int record_floats, cudaStream_t s) {
    using dev::Sample;
    if (in == Sample::f32 && out == Sample::f32)
        return plaunch_typed<HB, K, float, float>(jobs, count, blocks, threads, record_floats, s);
    if (in == Sample::u16 && out == Sample::f32)
        return plaunch_typed<HB, K, std::uint16_t, float>(jobs, count, blocks, threads, record_floats, s);
    if (in == Sample::u8 && out == Sample::f32)
        return plaunch_typed<HB, K, std::uint8_t, float>(jobs, count, blocks, threads, record_floats, s);
    if (in == Sample::f32 && out == Sample::u16)
        return plaunch_typed<HB, K, float, std::uint16_t>(jobs, count, blocks, threads, record_floats, s);
    if (in == Sample::f32 && out == Sample::u8)
        return plaunch_typed<HB, K, float, std::uint8_t>(jobs, count, blocks, threads, record_floats, s);
    return static_cast<int>(cudaErrorInvalidValue);
}

} // namespace
} // namespace dsmvc_gb
