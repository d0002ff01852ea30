// Two-pass transposing kernels: the exact 2D passes of a Float32 descale.
//
// The same warp layout, ring feeding and record staging as the chunk-delayed
// transposing kernels (tstream_impl.cuh), but the substitution runs as two
// sweeps over the vector:
//
//  * forward sweep, first destination to last: the gather and the forward
//    substitution in the reference CUDA order, each forward value stored to
//    a Float32 plane laid out like the output (destination-major, the warp's
//    32 vectors adjacent: one coalesced store);
//  * backward sweep, last chunk to first: the chunk's 32 forward values of
//    each lane loaded at once (coalesced), the backward substitution in the
//    reference order from the exact carry of the chunk after it, each result
//    stored as soon as it is known.
//
// Nothing is approximated, so the results equal the reference CUDA kernels'
// bit for bit, for any decay of the factors and half-bandwidths up to 11.
// The ring is refilled per destination (windows up to 16 samples), or per
// group of four destinations for window 8 where the host's replay admits it.
// The forward plane is the output itself where it is a Float32 plane with
// the output's layout (the first pass's intermediate, Float32 outputs), else
// a caller scratch plane.  Registers hold one chunk at a time.
#pragma once

#include "tstream_impl.cuh"

namespace dsmvc_gb {
namespace {

template <int HB, int K, class In, class Out>
__global__ void __launch_bounds__(kTMaxThreads)
tsolve_kernel(const StreamJob *__restrict__ jobs, int job_count, int record_floats) {
    constexpr int LC = kTChunk;
    extern __shared__ __align__(16) float smem[];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nthreads = static_cast<int>(blockDim.x);
    // Jobs are assigned warps; a CTA's warps share one plan.
    const int cta_warp = static_cast<int>(blockIdx.x) * (nthreads >> 5);
    const StreamJob &job = jobs[find_tjob(jobs, job_count, cta_warp + warp)];
    const StreamJob &lead = jobs[find_tjob(jobs, job_count, cta_warp)];
    const dev::StreamPlanView p = lead.plan;
    const int n = p.destination_size;
    const int chunks = (n + LC - 1) / LC;
    // Chunks stored: [ca, cb); a segment (chunk_end > 0) sweeps forward over
    // [fc0, fce] from a zero history and backward from a zero carry after
    // fce, `margin` chunks beyond its range on either side (within the
    // vector), with its forward values in its own region from chunk fc0 on.
    // Every warp of a CTA serves the same plan and range.
    const bool segment = lead.chunk_end > 0;
    const int ca = lead.chunk_begin;
    const int cb = segment ? lead.chunk_end : chunks;
    const int fc0 = segment ? max(ca - lead.margin, 0) : 0;
    const int fce = segment ? min(cb + lead.margin, chunks) - 1 : chunks - 1;
    const int ybase = fc0 * LC;
    const int per_buffer = kTChunk * record_floats;
    float *bufs = smem;
    float *ring = smem + 3 * per_buffer + warp * kTRingFloats;

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

    WarpFeeder<In, false> feed;
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

    // Forward value of destination j at yplane[j * y_elem] (a segment's
    // region starts at its first computed destination).
    float *yplane = job.y + v - static_cast<std::int64_t>(ybase) * job.y_elem;
    Out *out = static_cast<Out *>(job.out) + v;
    const int fs = fwd_stride<HB, K>(p), bs = bwd_stride<HB, K>(p);
    const int kw = K > 0 ? K : p.window;

    // ---- forward sweep ---------------------------------------------------
    tstage(bufs + (fc0 % 3) * per_buffer, p, fc0, tid, nthreads);
    tcp_commit();
    if (fc0 + 1 <= fce) tstage(bufs + ((fc0 + 1) % 3) * per_buffer, p, fc0 + 1, tid, nthreads);
    tcp_commit();
    float hist[HB];
#pragma unroll
    for (int d = 0; d < HB; ++d) hist[d] = 0.0f;
    for (int c = fc0; c <= fce; ++c) {
        tcp_wait_one();
        __syncthreads();
        const float *fwd = bufs + (c % 3) * per_buffer;
        const int j0 = c * LC;
        if (!idle) {
            float y[LC];
#pragma unroll
            for (int t = 0; t < LC; ++t) {
                if constexpr (K > 0) {
                    // Window 8: one refill per group of four destinations.
                    if (t % 4 == 0) {
                        const int s_last = __float_as_int(fwd[(t + 3) * fs]);
                        const int need = max(s_last, __float_as_int(fwd[t * fs])) + kw;
                        feed.ensure(min(need, p.source_size));
                    }
                }
                const float *rec = fwd + t * fs;
                const float4 hdr = tlds4(rec);
                if constexpr (K == 0) feed.ensure(min(__float_as_int(hdr.x) + kw, p.source_size));
                const float *win = feed.ring + lane + __float_as_int(hdr.z);
                float sum = 0.0f;
                if constexpr (K > 0) {
#pragma unroll
                    for (int k = 0; k < K; k += 4) {
                        const float4 w = tlds4(rec + 4 + k);
                        sum = fmaf(w.x, win[(k + 0) * kTPitch], sum);
                        sum = fmaf(w.y, win[(k + 1) * kTPitch], sum);
                        sum = fmaf(w.z, win[(k + 2) * kTPitch], sum);
                        sum = fmaf(w.w, win[(k + 3) * kTPitch], sum);
                    }
                } else {
                    for (int k = 0; k < kw; k += 4) {
                        const float4 w = tlds4(rec + 4 + k);
                        sum = fmaf(w.x, win[(k + 0) * kTPitch], sum);
                        sum = fmaf(w.y, win[(k + 1) * kTPitch], sum);
                        sum = fmaf(w.z, win[(k + 2) * kTPitch], sum);
                        sum = fmaf(w.w, win[(k + 3) * kTPitch], sum);
                    }
                }
                const float *low = rec + 4 + kw;
#pragma unroll
                for (int q = 0; q < HB; q += 4) {
                    const float4 l = tlds4(low + q);
                    const float lv[4] = {l.x, l.y, l.z, l.w};
#pragma unroll
                    for (int e = 0; e < 4; ++e) {
                        const int d = HB - (q + e);
                        if (d >= 1) {
                            const float prev = t - d >= 0 ? y[t - d >= 0 ? t - d : 0] : hist[t - d < 0 ? HB + t - d : 0];
                            sum = fmaf(lv[e], prev, sum);
                        }
                    }
                }
                y[t] = j0 + t < n ? sum * hdr.y : 0.0f;
                if (active && j0 + t < n) yplane[static_cast<std::int64_t>(j0 + t) * job.y_elem] = y[t];
            }
#pragma unroll
            for (int d = 0; d < HB; ++d) hist[d] = y[LC - HB + d];
        }
        __syncthreads();
        if (c + 2 <= fce) tstage(bufs + ((c + 2) % 3) * per_buffer, p, c + 2, tid, nthreads);
        tcp_commit();
    }

    // ---- backward sweep --------------------------------------------------
    asm volatile("cp.async.wait_all;\n" ::: "memory");
    __syncthreads();
    tstage(bufs, p, fce, tid, nthreads);
    tcp_commit();
    if (fce - 1 >= ca) tstage(bufs + per_buffer, p, fce - 1, tid, nthreads);
    tcp_commit();
    float carry[HB];
#pragma unroll
    for (int d = 0; d < HB; ++d) carry[d] = 0.0f;
    for (int c = fce, k = 0; c >= ca; --c, ++k) {
        const int j0 = c * LC;
        const bool store = active && c < cb;
        float yv[LC];
        if (!idle) {
#pragma unroll
            for (int t = 0; t < LC; ++t)
                yv[t] = (active && j0 + t < n) ? yplane[static_cast<std::int64_t>(j0 + t) * job.y_elem] : 0.0f;
        }
        tcp_wait_one();
        __syncthreads();
        const float *bwd = bufs + (k % 3) * per_buffer + kTChunk * fs;
        if (!idle) {
            float x[HB];                                  // x[(t + d) % HB] = x_{t + d} of the chunk
#pragma unroll
            for (int t = LC - 1; t >= 0; --t) {
                const float *rec = bwd + t * bs;
                float sum = 0.0f;
#pragma unroll
                for (int q = 0; q < HB; q += 4) {
                    const float4 u = tlds4(rec + q);
                    const float uv[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
                    for (int e = 0; e < 4; ++e) {
                        const int pos = q + e;
                        if (pos < HB) {
                            const int d = HB == 3 ? pos + 1 : HB - pos;
                            const float xd = (t + d < LC) ? x[(t + d) % HB] : carry[t + d >= LC ? t + d - LC : 0];
                            sum = fmaf(uv[e], xd, sum);
                        }
                    }
                }
                const float xt = yv[t] - sum;
                x[t % HB] = xt;
                if (store && j0 + t < n) out[static_cast<std::int64_t>(j0 + t) * job.out_elem] = tout<Out>(xt, job.conv);
            }
#pragma unroll
            for (int d = 0; d < HB; ++d) carry[d] = x[d];
        }
        __syncthreads();
        if (c - 2 >= ca) tstage(bufs + ((k + 2) % 3) * per_buffer, p, c - 2, tid, nthreads);
        tcp_commit();
    }
}

template <int HB, int K, class In, class Out>
int xlaunch_typed(const StreamJob *jobs, int count, int blocks, int threads, int record_floats, cudaStream_t s) {
    if (threads < 32 || threads > kTMaxThreads || threads % 32) return static_cast<int>(cudaErrorInvalidValue);
    const int smem = (3 * kTChunk * record_floats + threads / 32 * kTRingFloats) * static_cast<int>(sizeof(float));
    auto kernel = tsolve_kernel<HB, K, In, Out>;
    static SmemLimit limit;
    if (const cudaError_t e = limit.ensure(kernel, smem); e != cudaSuccess) return static_cast<int>(e);
    kernel<<<blocks, threads, smem, s>>>(jobs, count, record_floats);
    return static_cast<int>(cudaGetLastError());
}

template <int HB, int K>
int xlaunch_k(const StreamJob *jobs, int count, int blocks, int threads, dev::Sample in, dev::Sample out,
              int record_floats, cudaStream_t s) {
    using dev::Sample;
    if (in == Sample::f32 && out == Sample::f32)
        return xlaunch_typed<HB, K, float, float>(jobs, count, blocks, threads, record_floats, s);
    if (in == Sample::u16 && out == Sample::f32)
        return xlaunch_typed<HB, K, std::uint16_t, float>(jobs, count, blocks, threads, record_floats, s);
    if (in == Sample::u8 && out == Sample::f32)
        return xlaunch_typed<HB, K, std::uint8_t, float>(jobs, count, blocks, threads, record_floats, s);
    if (in == Sample::f32 && out == Sample::u16)
        return xlaunch_typed<HB, K, float, std::uint16_t>(jobs, count, blocks, threads, record_floats, s);
    if (in == Sample::f32 && out == Sample::u8)
        return xlaunch_typed<HB, K, float, std::uint8_t>(jobs, count, blocks, threads, record_floats, s);
    return static_cast<int>(cudaErrorInvalidValue);
}

} // namespace
} // namespace dsmvc_gb
