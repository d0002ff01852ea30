// Streaming axis kernels: one thread per vector (row or column), the vector
// walked once from its first to its last sample.
//
//  * Source samples stream through a per-thread ring in shared memory
//    (32 samples, stored twice so that any window of up to 32 consecutive
//    samples is contiguous).  Each lane reads and writes only its own ring
//    column.  Rows are fetched with 16-byte vector loads, columns with one
//    coalesced load per source row for the warp; the next block is always in
//    flight while the current one is consumed.
//  * Per-destination records (window start, zero-padded A^T weights, forward
//    factors, inverse diagonal; backward factors) are copied a chunk of 32
//    destinations at a time into the warp's shared memory with cp.async,
//    three chunk buffers deep, two chunks ahead of use.  Every lane of a warp
//    works on the same destination, so record reads are broadcasts.
//  * Weights apply in ascending source order (zero weights are exact no-ops),
//    so the forward substitution is the reference CUDA operation order bit
//    for bit.
//  * The forward results of two chunks live in registers.  The backward
//    substitution of chunk c starts from the end of chunk c+1 with a zero
//    carry: after one chunk the carry's influence is below 2^-26 per slot (the
//    host admits a plan only when that holds for every chunk), so the state
//    entering chunk c equals the true one to within rounding and no forward
//    value is written to memory.  The last chunk's backward pass is exact.
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

constexpr int kRing = kStreamRing;   // samples held per thread
constexpr int kChunk = kStreamChunk; // destinations per record chunk
constexpr int kThreads = 128;
constexpr int kWarps = kThreads / 32;
constexpr int kRingFloats = 2 * kRing * 32;   // per warp

__device__ __forceinline__ int find_stream_job(const StreamJob *jobs, int count, int block) {
    int lo = 0, hi = count - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (jobs[mid].first_block <= block) lo = mid; else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ void cp_async16(float *smem, const float *gmem) {
    const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" :: "r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_one() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }

template <class T> __device__ __forceinline__ float to_f32(T v, const Conversion &c) {
    return (static_cast<float>(v) - c.in_offset) * c.in_scale;
}
template <> __device__ __forceinline__ float to_f32<float>(float v, const Conversion &) { return v; }

template <class T> __device__ __forceinline__ T from_f32(float v, const Conversion &c) {
    float s = __fadd_rn(__fmul_rn(v, c.out_scale), c.out_offset);
    s = fminf(fmaxf(s, 0.0f), static_cast<float>(c.out_max));
    return static_cast<T>(__float2uint_rn(s));
}
template <> __device__ __forceinline__ float from_f32<float>(float v, const Conversion &) { return v; }

// Loads source samples into the ring, one block ahead of use.
template <class In, bool CONTIG>
struct Feeder {
    static constexpr int V = CONTIG ? 16 / static_cast<int>(sizeof(In)) : 4;
    const In *base;          // this thread's vector
    std::int64_t elem;       // element stride (CONTIG: 1)
    int size;                // source samples in the vector
    int have;                // samples in the ring
    bool pend_ok;            // `pend` holds samples [have, have + V)
    bool vec_ok;             // CONTIG: 16-byte aligned row
    float *ring;             // this lane's ring column (stride 32 floats)
    Conversion conv;
    uint4 pend_raw;          // CONTIG pending block
    In pend[4];              // strided pending rows

    __device__ __forceinline__ void put(int s, float x) {
        const int r = (s & (kRing - 1)) * 32;
        ring[r] = x;
        ring[r + kRing * 32] = x;
    }

    __device__ __forceinline__ void issue() {
        pend_ok = have + V <= size && (!CONTIG || vec_ok);
        if (!pend_ok) return;
        if constexpr (CONTIG) {
            pend_raw = __ldg(reinterpret_cast<const uint4 *>(base + have));
        } else {
#pragma unroll
            for (int k = 0; k < 4; ++k) pend[k] = __ldg(base + (have + k) * elem);
        }
    }

    __device__ __forceinline__ void start() {
        have = 0;
        issue();
    }

    // Ensures samples [0, need) are in the ring (need <= size).
    __device__ __forceinline__ void ensure(int need) {
        while (have < need) {
            if (pend_ok) {
                if constexpr (CONTIG) {
                    const In *vals = reinterpret_cast<const In *>(&pend_raw);
#pragma unroll
                    for (int k = 0; k < V; ++k) put(have + k, to_f32(vals[k], conv));
                } else {
#pragma unroll
                    for (int k = 0; k < 4; ++k) put(have + k, to_f32(pend[k], conv));
                }
                have += V;
                issue();
            } else {
                put(have, to_f32(__ldg(base + have * elem), conv));
                have += 1;
            }
        }
    }
};

// One chunk of records in shared memory: forward[32][fs], backward[32][bs].
struct ChunkRecords {
    const float *fwd;
    const float *bwd;
};

__device__ __forceinline__ void stage_chunk(float *buf, const dev::StreamPlanView &p, int chunk, int lane) {
    const int fs = p.forward_stride, bs = p.backward_stride;
    const float *gf = p.forward + static_cast<std::int64_t>(chunk) * kChunk * fs;
    const float *gb = p.backward + static_cast<std::int64_t>(chunk) * kChunk * bs;
    for (int i = lane * 4; i < kChunk * fs; i += 128) cp_async16(buf + i, gf + i);
    float *bb = buf + kChunk * fs;
    for (int i = lane * 4; i < kChunk * bs; i += 128) cp_async16(bb + i, gb + i);
}

__device__ __forceinline__ float4 lds4(const float *p) { return *reinterpret_cast<const float4 *>(p); }

// Forward substitution of destinations [j0, j0 + LC) into y[LC + t]; the
// preceding chunk's values are in y[0, LC) (zeros before the first one).
template <int HB, int LC, class Feed>
__device__ __forceinline__ void forward_chunk(float (&y)[2 * LC], int j0, const dev::StreamPlanView &p,
                                              const ChunkRecords &r, Feed &feed) {
    const int K = p.window;
    const int fs = p.forward_stride;
#pragma unroll
    for (int t = 0; t < LC; ++t) {
        if (j0 + t >= p.destination_size) {
            y[LC + t] = 0.0f;
            continue;
        }
        const float *rec = r.fwd + t * fs;
        const float4 hdr = lds4(rec);
        const int s0 = __float_as_int(hdr.x);
        feed.ensure(s0 + K);
        const float *win = feed.ring + (s0 & (kRing - 1)) * 32;
        float sum = 0.0f;
        for (int k = 0; k < K; k += 4) {
            const float4 w = lds4(rec + 4 + k);
            sum = fmaf(w.x, win[(k + 0) * 32], sum);
            sum = fmaf(w.y, win[(k + 1) * 32], sum);
            sum = fmaf(w.z, win[(k + 2) * 32], sum);
            sum = fmaf(w.w, win[(k + 3) * 32], sum);
        }
        // Factors stored negated in use order d = HB..1 (zero where d > j).
        const float *low = rec + 4 + K;
#pragma unroll
        for (int q = 0; q < HB; q += 4) {
            const float4 l = lds4(low + q);
            const float lv[4] = {l.x, l.y, l.z, l.w};
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const int d = HB - (q + e);
                if (d >= 1) sum = fmaf(lv[e], y[LC + t - d], sum);
            }
        }
        y[LC + t] = sum * hdr.y;
    }
}

// Backward substitution of destinations [j0, j0 + LC) held in y[B + t],
// in place (y -> x).  carry[e] holds x_{j0+LC+e} on entry and x_{j0+e} on
// exit.
template <int HB, int LC, int B>
__device__ __forceinline__ void backward_chunk(float (&y)[2 * LC], float (&carry)[HB], int j0,
                                               const dev::StreamPlanView &p, const float *bwd) {
    const int bs = p.backward_stride;
#pragma unroll
    for (int t = LC - 1; t >= 0; --t) {
        if (j0 + t >= p.destination_size) continue;
        const float *rec = bwd + t * bs;
        float sum = 0.0f;
#pragma unroll
        for (int q = 0; q < HB; q += 4) {
            const float4 u = lds4(rec + q);
            const float uv[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const int pos = q + e;
                if (pos < HB) {
                    const int d = HB == 3 ? pos + 1 : HB - pos;
                    const float xd = (t + d < LC) ? y[B + (t + d < LC ? t + d : 0)]
                                                  : carry[t + d >= LC ? t + d - LC : 0];
                    sum = fmaf(uv[e], xd, sum);
                }
            }
        }
        y[B + t] = y[B + t] - sum;
    }
#pragma unroll
    for (int d = 0; d < HB; ++d) carry[d] = y[B + d];
}

// Zero-carry backward warm-up over the chunk in y[LC, 2 LC): only the state
// entering the preceding chunk is kept (in `carry`); y is untouched.
template <int HB, int LC>
__device__ __forceinline__ void warmup_chunk(const float (&y)[2 * LC], float (&carry)[HB], int j0,
                                             const dev::StreamPlanView &p, const float *bwd) {
    const int bs = p.backward_stride;
    float w[HB];   // x_t lives in w[t % HB]
#pragma unroll
    for (int t = LC - 1; t >= 0; --t) {
        float sum = 0.0f;
        if (j0 + t < p.destination_size) {
            const float *rec = bwd + t * bs;
#pragma unroll
            for (int q = 0; q < HB; q += 4) {
                const float4 u = lds4(rec + q);
                const float uv[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    const int pos = q + e;
                    if (pos < HB) {
                        const int d = HB == 3 ? pos + 1 : HB - pos;
                        const float xd = (t + d < LC) ? w[(t + d) % HB]
                                                      : carry[t + d >= LC ? t + d - LC : 0];
                        sum = fmaf(uv[e], xd, sum);
                    }
                }
            }
        }
        w[t % HB] = y[LC + t] - sum;
    }
#pragma unroll
    for (int d = 0; d < HB; ++d) carry[d] = w[d];
}

template <class Out, bool CONTIG, int LC, int B>
__device__ __forceinline__ void emit_chunk(const float (&y)[2 * LC], int j0, Out *out,
                                           std::int64_t elem, int n, bool vec_ok, bool active,
                                           const Conversion &conv) {
    if (!active) return;
    if constexpr (CONTIG && sizeof(Out) == 4) {
        if (vec_ok && j0 + LC <= n) {
#pragma unroll
            for (int t = 0; t < LC; t += 4) {
                const float4 v = make_float4(y[B + t], y[B + t + 1], y[B + t + 2], y[B + t + 3]);
                *reinterpret_cast<float4 *>(out + j0 + t) = v;
            }
            return;
        }
    }
#pragma unroll
    for (int t = 0; t < LC; ++t) {
        const int j = j0 + t;
        if (j < n) out[static_cast<std::int64_t>(j) * elem] = from_f32<Out>(y[B + t], conv);
    }
}

// y[0, LC) holds chunk c-1 and y[LC, 2 LC) chunk c: the forward pass fills
// the upper half, the lower half is finished by a backward pass that starts
// from the upper half's warm-up (or, for the last chunk, from the exact end
// of the vector), and the upper half then moves down.  Every lane of the
// warp runs the whole loop (lanes past the last vector compute on a clamped
// vector and store nothing), because the record copies are shared.
template <int HB, int LC, class In, class Out, bool CONTIG>
__global__ void __launch_bounds__(kThreads)
stream_kernel(const StreamJob *__restrict__ jobs, int job_count, int records_per_buffer) {
    static_assert(LC == kChunk, "record chunks and register chunks coincide");
    extern __shared__ __align__(16) float smem[];
    const int jidx = find_stream_job(jobs, job_count, static_cast<int>(blockIdx.x));
    const StreamJob &job = jobs[jidx];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int first = (static_cast<int>(blockIdx.x) - job.first_block) * kThreads + warp * 32;
    if (first >= job.vectors) return;                 // whole warp idle
    const int v_raw = first + lane;
    const bool active = v_raw < job.vectors;
    const int v = active ? v_raw : job.vectors - 1;
    const dev::StreamPlanView p = job.plan;
    const int n = p.destination_size;

    float *wsm = smem + warp * (kRingFloats + 3 * records_per_buffer);
    float *bufs = wsm + kRingFloats;
    const int buf_floats = records_per_buffer;

    Feeder<In, CONTIG> feed;
    feed.base = static_cast<const In *>(job.in) + v * job.in_vec;
    feed.elem = job.in_elem;
    feed.size = p.source_size;
    feed.conv = job.conv;
    feed.vec_ok = CONTIG && (reinterpret_cast<std::uintptr_t>(feed.base) % 16 == 0);
    feed.ring = wsm + lane;
    feed.start();

    Out *out = static_cast<Out *>(job.out) + v * job.out_vec;
    const bool out_vec_ok = CONTIG && (reinterpret_cast<std::uintptr_t>(out) % 16 == 0);

    const int chunks = (n + LC - 1) / LC;
    stage_chunk(bufs, p, 0, lane);
    cp_async_commit();
    if (chunks > 1) stage_chunk(bufs + buf_floats, p, 1, lane);
    cp_async_commit();

    float y[2 * LC];
    float carry[HB];
#pragma unroll
    for (int t = 0; t < LC; ++t) y[t] = 0.0f;
    for (int c = 0; c < chunks; ++c) {
        cp_async_wait_one();
        __syncwarp();
        float *cur = bufs + (c % 3) * buf_floats;
        float *prev = bufs + ((c + 2) % 3) * buf_floats;
        const ChunkRecords rc{cur, cur + kChunk * p.forward_stride};
        forward_chunk<HB, LC>(y, c * LC, p, rc, feed);
        const bool last = c + 1 == chunks;
#pragma unroll
        for (int d = 0; d < HB; ++d) carry[d] = 0.0f;
        if (last) {
            backward_chunk<HB, LC, LC>(y, carry, c * LC, p, rc.bwd);
            emit_chunk<Out, CONTIG, LC, LC>(y, c * LC, out, job.out_elem, n, out_vec_ok, active, job.conv);
        } else {
            warmup_chunk<HB, LC>(y, carry, c * LC, p, rc.bwd);
        }
        if (c > 0) {
            backward_chunk<HB, LC, 0>(y, carry, (c - 1) * LC, p, prev + kChunk * p.forward_stride);
            emit_chunk<Out, CONTIG, LC, 0>(y, (c - 1) * LC, out, job.out_elem, n, out_vec_ok, active,
                                           job.conv);
        }
        if (last) return;
        // The buffer of chunk c-1 is free: fetch chunk c+2 into it.
        __syncwarp();
        if (c + 2 < chunks) stage_chunk(prev, p, c + 2, lane);
        cp_async_commit();
#pragma unroll
        for (int t = 0; t < LC; ++t) y[t] = y[LC + t];
    }
}

template <int HB, int LC, class In, class Out, bool CONTIG>
int launch_typed(const StreamJob *jobs, int count, int blocks, int record_floats, cudaStream_t s) {
    const int per_buffer = kChunk * record_floats;
    const int smem = kWarps * (kRingFloats + 3 * per_buffer) * static_cast<int>(sizeof(float));
    auto kernel = stream_kernel<HB, LC, In, Out, CONTIG>;
    static SmemLimit limit;
    if (const cudaError_t e = limit.ensure(kernel, smem); e != cudaSuccess) return static_cast<int>(e);
    kernel<<<blocks, kThreads, smem, s>>>(jobs, count, per_buffer);
    return static_cast<int>(cudaGetLastError());
}

template <int HB, int LC>
int launch_hb(const StreamJob *jobs, int count, int blocks, bool contig, dev::Sample in,
              dev::Sample out, int record_floats, cudaStream_t s) {
    using dev::Sample;
    if (contig) {
        if (out != Sample::f32) return static_cast<int>(cudaErrorInvalidValue);
        if (in == Sample::f32) return launch_typed<HB, LC, float, float, true>(jobs, count, blocks, record_floats, s);
        if (in == Sample::u16) return launch_typed<HB, LC, std::uint16_t, float, true>(jobs, count, blocks, record_floats, s);
        if (in == Sample::u8) return launch_typed<HB, LC, std::uint8_t, float, true>(jobs, count, blocks, record_floats, s);
    } else {
        if (in != Sample::f32) return static_cast<int>(cudaErrorInvalidValue);
        if (out == Sample::f32) return launch_typed<HB, LC, float, float, false>(jobs, count, blocks, record_floats, s);
        if (out == Sample::u16) return launch_typed<HB, LC, float, std::uint16_t, false>(jobs, count, blocks, record_floats, s);
        if (out == Sample::u8) return launch_typed<HB, LC, float, std::uint8_t, false>(jobs, count, blocks, record_floats, s);
    }
    return static_cast<int>(cudaErrorInvalidValue);
}

} // namespace
} // namespace dsmvc_gb
