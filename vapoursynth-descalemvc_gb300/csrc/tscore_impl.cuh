// Columns pass of a sweep candidate's 2D descale with its scoring fused in
// (dev::ScoreEpilogue, score.cuh): the chunk-delayed transposing kernel of
// tstream_impl.cuh (Float32 intermediate in, the same records, ring feeder
// and substitutions, so every descaled value is bit for bit the one the
// unfused pass stores), whose results go to shared memory instead of HBM.
//
//  * A CTA of kScoreCtaThreads threads (8 warps) serves one tile of the
//    candidate's descaled columns, 256 from the tile's origin; neighbouring
//    tiles overlap by about the horizontal operator's window.
//  * Each lane keeps its column's last kScoreRingRows descaled rows (the
//    chunk just finished and the 6 rows before it) in a lane-private ring.
//  * After each chunk, the source rows whose vertical window ends in it are
//    re-upscaled in batches of kScoreBatchRows: every warp applies the
//    vertical operator to its 32 columns into a shared row buffer (the
//    tile's columns, then 8 zero columns), and after a barrier every thread
//    applies the horizontal operator for the tile's source columns and sums
//    |re-upscaled - frame| (float per batch, double across batches).
//  * At the end the CTA's sums reduce in a fixed order into the tile's
//    partial; launch_fused_score_finalize adds the tiles in order.  A score
//    depends only on the candidate, never on the launch it shares.
#pragma once

#include "score.cuh"
#include "tstream_impl.cuh"

namespace dsmvc_gb {
namespace {

constexpr int kFWarps = kScoreCtaThreads / 32;
constexpr int kFHalo = kScoreRingRows - kTChunk;          // rows kept before the chunk
constexpr int kFPitch = kScoreCtaThreads + 8;             // row buffer pitch (floats)
static_assert(kFHalo >= kScoreMaxVerticalTaps - 1, "the ring holds every window of the chunk's rows");
static_assert(kFPitch - kScoreCtaThreads >= kScoreMaxHorizontalTaps - 1, "zero columns cover padded windows");

// Backward substitution of the chunk in y[B, B + LC) from `carry`, as
// tbackward (tstream_impl.cuh) without the stores: the chunk's x values stay
// in y[B, B + LC).
template <int HB, int LC, int K, int B>
__device__ __forceinline__ void tbackward_keep(float (&y)[2 * LC], float (&carry)[HB], const dev::StreamPlanView &p,
                                               const float *bwd) {
    const int bs = bwd_stride<HB, K>(p);
    TBackCoeffs<HB, K> u;
#pragma unroll
    for (int t = LC - 1; t >= 0; --t) {
        u.at(bwd, bs, t);
        float sum = 0.0f;
#pragma unroll
        for (int pos = 0; pos < HB; ++pos) {
            const int d = HB == 3 ? pos + 1 : HB - pos;
            const float xd = (t + d < LC) ? y[B + (t + d < LC ? t + d : 0)]
                                          : carry[t + d >= LC ? t + d - LC : 0];
            sum = fmaf(u(t, pos), xd, sum);
        }
        y[B + t] = y[B + t] - sum;
    }
#pragma unroll
    for (int d = 0; d < HB; ++d) carry[d] = y[B + d];
}

// Moves the previous chunk's last kFHalo rows to the front of the lane's
// ring and puts the chunk y[B, B + LC) after them: slot i then holds
// descaled row 32 q - kFHalo + i for chunk q.
template <int LC, int B>
__device__ __forceinline__ void ring_put(float *dr, const float (&y)[2 * LC]) {
#pragma unroll
    for (int i = 0; i < kFHalo; ++i) dr[i * 32] = dr[(LC + i) * 32];
#pragma unroll
    for (int t = 0; t < LC; ++t) dr[(kFHalo + t) * 32] = y[B + t];
}

// The CTA's tile, in shared memory (read where needed, so that it holds no
// registers across the substitutions).
struct FusedTile {
    const dev::ScoreEpilogue *ep;
    int c_lo;             // the tile's first descaled column
    int s_begin, s_end;   // the tile's source columns
};

// Copies the vertical records of source rows [rb, rb + nb) into `rec`
// (kScoreBatchRows x 12 floats): one 16-byte copy per thread.
__device__ __forceinline__ void stage_rows(float *rec, const float *v_rows, int rb, int nb) {
    const int t = static_cast<int>(threadIdx.x);
    if (t < nb * 3)
        reinterpret_cast<float4 *>(rec)[t] = __ldg(reinterpret_cast<const float4 *>(v_rows + static_cast<std::int64_t>(rb) * 12) + t);
}

// Re-upscales and scores the source rows emitted after chunk q into `err`.
// Every thread of the CTA calls it with the same q (it holds barriers).
// `dr`: the lane's ring column; `vb`: the row buffer; `vrec`: two batches
// of vertical records; `col_ok`: the thread's descaled column (warp * 32 +
// lane of the tile) exists.
__device__ __forceinline__ void fused_emit(const FusedTile &f, float *dr, float *vb, float *vrec, bool col_ok,
                                           double &err, int q) {
    const dev::ScoreEpilogue &ep = *f.ep;
    const int tid = static_cast<int>(threadIdx.x);
    const int r_begin = q > 0 ? __ldg(ep.v_emit + q - 1) : 0;
    const int r_end = __ldg(ep.v_emit + q);
    if (r_begin >= r_end) return;
    const int slot_row0 = q * kTChunk - kFHalo;
    const int vt = ep.v_taps, ht = ep.h_taps;
    stage_rows(vrec, ep.v_rows, r_begin, min(kScoreBatchRows, r_end - r_begin));
    __syncthreads();
    int buf = 0;
    const int c_lo = f.c_lo, s_end = f.s_end, s_first = f.s_begin + tid;
    for (int rb = r_begin; rb < r_end; rb += kScoreBatchRows, buf ^= 1) {
        const int nb = min(kScoreBatchRows, r_end - rb);
        const float *rec = vrec + buf * (kScoreBatchRows * 12);
        // The frame rows of this thread's first source column, in flight
        // during the vertical operator and the barrier.
        float fv[kScoreBatchRows];
        const float *fr = ep.frame + static_cast<std::int64_t>(rb) * ep.frame_stride;
#pragma unroll
        for (int i = 0; i < kScoreBatchRows; ++i)
            fv[i] = i < nb && s_first < s_end ? __ldg(fr + i * ep.frame_stride + s_first) : 0.0f;
        // Vertical operator: rows rb .. rb + nb of this lane's column (even
        // and odd taps in two sums).
#pragma unroll
        for (int i = 0; i < kScoreBatchRows; ++i) {
            if (i < nb) {
                const float *ri = rec + i * 12;
                const float *d = dr + (__float_as_int(ri[0]) - slot_row0) * 32;
                float a0 = 0.0f, a1 = 0.0f;
                for (int e = 0; e < vt; e += 4) {
                    const float4 w = *reinterpret_cast<const float4 *>(ri + 4 + e);
                    a0 = fmaf(w.x, d[(e + 0) * 32], a0);
                    a1 = fmaf(w.y, d[(e + 1) * 32], a1);
                    a0 = fmaf(w.z, d[(e + 2) * 32], a0);
                    a1 = fmaf(w.w, d[(e + 3) * 32], a1);
                }
                vb[i * kFPitch + tid] = col_ok ? a0 + a1 : 0.0f;
            }
        }
        __syncthreads();
        // The next batch's records, while the row buffer is consumed.
        if (rb + kScoreBatchRows < r_end)
            stage_rows(vrec + (buf ^ 1) * (kScoreBatchRows * 12), ep.v_rows, rb + kScoreBatchRows,
                       min(kScoreBatchRows, r_end - rb - kScoreBatchRows));
        // Horizontal operator and the error sums of the tile's source columns.
        float sum = 0.0f;
        for (int s = s_first; s < s_end; s += kScoreCtaThreads) {
            const float4 *hr = reinterpret_cast<const float4 *>(ep.h_cols + static_cast<std::int64_t>(s) * 12);
            if (s != s_first) {
#pragma unroll
                for (int i = 0; i < kScoreBatchRows; ++i) fv[i] = i < nb ? __ldg(fr + i * ep.frame_stride + s) : 0.0f;
            }
            const float4 h0 = __ldg(hr);
            const float4 w0 = __ldg(hr + 1);
            const float4 w1 = ht > 4 ? __ldg(hr + 2) : make_float4(0, 0, 0, 0);
            const float *v = vb + (__float_as_int(h0.x) - c_lo);
#pragma unroll
            for (int i = 0; i < kScoreBatchRows; ++i) {
                if (i < nb) {
                    const float *vr = v + i * kFPitch;
                    float a0 = 0.0f, a1 = 0.0f;
                    a0 = fmaf(w0.x, vr[0], a0);
                    a1 = fmaf(w0.y, vr[1], a1);
                    a0 = fmaf(w0.z, vr[2], a0);
                    a1 = fmaf(w0.w, vr[3], a1);
                    if (ht > 4) {
                        a0 = fmaf(w1.x, vr[4], a0);
                        a1 = fmaf(w1.y, vr[5], a1);
                        a0 = fmaf(w1.z, vr[6], a0);
                        a1 = fmaf(w1.w, vr[7], a1);
                    }
                    sum += fabsf((a0 + a1) - fv[i]);
                }
            }
        }
        err += static_cast<double>(sum);
        __syncthreads();
    }
}

// At most 168 registers a thread: three CTAs (12 warps) per SM.
template <int HB, int LC, int K>
__global__ void __launch_bounds__(kScoreCtaThreads, 3)
tscore_kernel(const StreamJob *__restrict__ jobs, int job_count, int record_floats) {
    static_assert(LC == kTChunk, "record chunks and register chunks coincide");
    extern __shared__ __align__(16) float smem[];
    __shared__ double warp_err[kFWarps];
    __shared__ __align__(16) float vrec[2 * kScoreBatchRows * 12];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    // Every job starts on a CTA: its tiles are its CTAs.
    const int cta_warp = static_cast<int>(blockIdx.x) * kFWarps;
    const StreamJob &job = jobs[find_tjob(jobs, job_count, cta_warp)];
    const dev::ScoreEpilogue *ep = static_cast<const dev::ScoreEpilogue *>(job.score);
    const dev::StreamPlanView p = job.plan;
    const int n = p.destination_size;
    const int chunks = (n + LC - 1) / LC;
    const int tile = (cta_warp - job.first_block) / kFWarps;
    const int per_buffer = kTChunk * record_floats;
    float *bufs = smem;
    float *ring = smem + 3 * per_buffer + warp * kTRingFloats;
    float *dring = smem + 3 * per_buffer + kFWarps * kTRingFloats + warp * (kScoreRingRows * 32);
    float *vb = smem + 3 * per_buffer + kFWarps * (kTRingFloats + kScoreRingRows * 32);

    __shared__ FusedTile f;
    if (tid == 0) {
        f.ep = ep;
        f.c_lo = ep->tile_origins[tile];
        f.s_begin = ep->tile_sources[tile];
        f.s_end = ep->tile_sources[tile + 1];
    }
    float *dr = dring + lane;
    double err = 0.0;

    int warp_first = ep->tile_origins[tile] + warp * 32;
    int warp_vectors = job.vectors - warp_first;
    const bool idle = warp_vectors <= 0;
    if (warp_vectors <= 0) {
        warp_first = job.vectors - 1;
        warp_vectors = 1;
    } else if (warp_vectors > 32) {
        warp_vectors = 32;
    }
    const bool col_ok = !idle && lane < warp_vectors;

    WarpFeeder<float, false> feed;
    feed.base = static_cast<const float *>(job.in) + warp_first * job.in_vec;
    feed.stride = job.in_vec;
    feed.size = p.source_size;
    feed.vectors = warp_vectors;
    feed.lane = lane;
    feed.ring = ring;
    feed.conv = job.conv;
    feed.vec_ok = (reinterpret_cast<std::uintptr_t>(job.in) % 16 == 0)
        && (job.in_vec * static_cast<std::int64_t>(sizeof(float))) % 16 == 0;
    if constexpr (K > 8) {
        for (int i = lane; i < kTRingFloats; i += 32) ring[i] = 0.0f;
        __syncwarp();
    }
    // Finite initial contents: the descaled-row ring (rows before the plane
    // and, in the last chunk, rows past it are read with zero weights) and
    // the row buffer (its zero columns are never written).
    for (int i = 0; i < kScoreRingRows; ++i) dr[i * 32] = 0.0f;
    for (int i = tid; i < kScoreBatchRows * kFPitch; i += kScoreCtaThreads) vb[i] = 0.0f;
    if (!idle) feed.start(0);

    const int ce = chunks - 1;
    tstage(bufs, p, 0, tid, kScoreCtaThreads);
    tcp_commit();
    if (1 <= ce) tstage(bufs + per_buffer, p, 1, tid, kScoreCtaThreads);
    tcp_commit();

    float y[2 * LC];
    float carry[HB];
#pragma unroll
    for (int t = 0; t < LC; ++t) y[t] = 0.0f;
    for (int c = 0;; ++c) {
        tcp_wait_one();
        __syncthreads();
        const float *cur = bufs + (c % 3) * per_buffer;
        const float *prev = bufs + ((c + 2) % 3) * per_buffer;
        const bool last = c + 1 == chunks;
        if (!idle) {
            if constexpr (K > 8) tforward_grouped<HB, LC, K>(y, cur, feed, lane);
            else tforward<HB, LC, K>(y, c * LC, p, cur, feed, lane);
            const float *cur_b = cur + kTChunk * fwd_stride<HB, K>(p);
            if (last) {
#pragma unroll
                for (int d = 0; d < HB; ++d) carry[d] = 0.0f;
                tbackward_keep<HB, LC, K, LC>(y, carry, p, cur_b);
            } else if (c > 0) {
                twarmup<HB, LC, K>(y, carry, p, cur_b);
            }
            if (c > 0) {
                tbackward_keep<HB, LC, K, 0>(y, carry, p, prev + kTChunk * fwd_stride<HB, K>(p));
                ring_put<LC, 0>(dr, y);
            }
        }
        if (c > 0) fused_emit(f, dr, vb, vrec, col_ok, err, c - 1);
        if (last) {
            if (!idle) ring_put<LC, LC>(dr, y);
            fused_emit(f, dr, vb, vrec, col_ok, err, c);
            break;
        }
        // Every warp is done with chunk c-1's records: fetch chunk c+2.
        __syncthreads();
        if (c + 2 <= ce) tstage(const_cast<float *>(prev), p, c + 2, tid, kScoreCtaThreads);
        tcp_commit();
#pragma unroll
        for (int t = 0; t < LC; ++t) y[t] = y[LC + t];
    }
    // The tile's partial: lanes, then warps, in a fixed order.
    double e = err;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) e += __shfl_down_sync(0xffffffffu, e, o);
    if (lane == 0) warp_err[warp] = e;
    __syncthreads();
    if (tid == 0) {
        double total = 0.0;
#pragma unroll
        for (int w = 0; w < kFWarps; ++w) total += warp_err[w];
        ep->partials[tile] = total;
    }
}

template <int HB, int K>
int tscore_launch(const StreamJob *jobs, int count, int blocks, int record_floats, cudaStream_t s) {
    const int smem = (3 * kTChunk * record_floats + kFWarps * (kTRingFloats + kScoreRingRows * 32)
                      + kScoreBatchRows * kFPitch) * static_cast<int>(sizeof(float));
    auto kernel = tscore_kernel<HB, kTChunk, K>;
    static SmemLimit limit;
    if (const cudaError_t e = limit.ensure(kernel, smem); e != cudaSuccess) return static_cast<int>(e);
    kernel<<<blocks, kScoreCtaThreads, smem, s>>>(jobs, count, record_floats);
    return static_cast<int>(cudaGetLastError());
}

// Windows 8 (compile-time gather), 12 / 16 (grouped records) and 0 (the
// plans' own window, looped).
template <int HB>
int tscore_launch_hb(const StreamJob *jobs, int count, int blocks, int window, int record_floats, cudaStream_t s) {
    switch (window) {
    case 0: return tscore_launch<HB, 0>(jobs, count, blocks, record_floats, s);
    case 8: return tscore_launch<HB, 8>(jobs, count, blocks, record_floats, s);
    case 12: return tscore_launch<HB, 12>(jobs, count, blocks, record_floats, s);
    case 16: return tscore_launch<HB, 16>(jobs, count, blocks, record_floats, s);
    default: return static_cast<int>(cudaErrorInvalidValue);
    }
}

} // namespace
} // namespace dsmvc_gb
