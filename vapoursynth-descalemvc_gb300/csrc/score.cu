// Candidate scoring kernels (score.cuh).
#include "score.cuh"
#include "smem_limit.cuh"

#include <cuda_runtime.h>

namespace dsmvc_gb {
namespace {

using dev::ScoreJob;

__device__ __forceinline__ int find_job(const ScoreJob *jobs, int count, int block) {
    int lo = 0, hi = count - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (jobs[mid].first_block <= block) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// Row-pass value of one column over one descaled row: its N entries
// (weights `w`, element offsets `c` from `y`) in ascending order.
template <int N>
__device__ __forceinline__ float tap_sum(const float *__restrict__ y, const float (&w)[8], const int (&c)[8]) {
    float acc = 0.0f;
#pragma unroll
    for (int e = 0; e < N; ++e) acc = fmaf(w[e], __ldg(y + c[e]), acc);
    return acc;
}

// The same for entries on consecutive columns y[0 .. N): immediate offsets.
template <int N>
__device__ __forceinline__ float tap_run(const float *__restrict__ y, const float (&w)[8]) {
    float acc = 0.0f;
#pragma unroll
    for (int e = 0; e < N; ++e) acc = fmaf(w[e], __ldg(y + e), acc);
    return acc;
}

// Row pass of one column over descaled rows [0, nj) from y (row stride ys)
// into z (stride kScoreThreads): `run` selects consecutive entries.
template <int N>
__device__ __forceinline__ void row_pass(float *z, const float *y, std::int64_t ys, int nj, bool run,
                                         const float (&w)[8], const int (&c)[8]) {
    // Four rows' loads in flight at a time.
    if (run) {

        for (int jj = 0; jj < nj; ++jj) z[jj * kScoreThreads] = tap_run<N>(y + jj * ys, w);
    } else {

        for (int jj = 0; jj < nj; ++jj) z[jj * kScoreThreads] = tap_sum<N>(y + jj * ys, w, c);
    }
}

// Column pass of one output row whose `count` entries (from `we`, each a
// (weight, byte offset) pair) sit on consecutive staged rows from byte
// offset `first` of this thread's column `zb`: immediate offsets.
template <int N>
__device__ __forceinline__ float col_run(const float2 *we, const char *zb) {
    float acc = 0.0f;
#pragma unroll
    for (int e = 0; e < N; ++e)
        acc = fmaf(we[e].x, *reinterpret_cast<const float *>(zb + e * kScoreThreads * 4), acc);
    return acc;
}

// Fused re-upscale and error sum of one column tile x one row segment of a
// candidate: the row-pass values Z[j][s] = sum_c A_h[s, c] Y[j][c] of the
// rows j the segment needs are computed into shared memory, then each
// source row r of the segment is sum_j A_v[r, j] Z[j][s], compared with the
// frame.  Errors are summed per block of kScoreRowBlock rows (each block's
// warp sums wait in shared memory; the segment's blocks are reduced
// together after its last, one barrier pair a segment).  Both passes
// run exact-length unrolled sums, with immediate offsets where a column's
// (row's) entries are consecutive, as they are away from the borders; the
// segment's A_v entries sit in shared memory as (weight, byte offset of the
// staged row) pairs with a per-row header (first entry, count, first
// offset, consecutive).  Every sum runs in ascending entry order.
__global__ void __launch_bounds__(kScoreThreads)
score_tiles_kernel(const ScoreJob *__restrict__ jobs, int count) {
    extern __shared__ float zt[];                  // [rows of the segment's span][kScoreThreads]
    constexpr int kWarps = kScoreThreads / 32, kPendingBlocks = 16;
    __shared__ float warp_sums[kPendingBlocks * kWarps];   // per pending row block, per warp
    __shared__ float2 seg_e[kScoreSegmentEntries]; // (weight, byte offset of the staged row, as bits)
    __shared__ int4 seg_r[kScoreMaxSegmentRows];   // (first entry, count, first offset, consecutive)
    __shared__ int span_lo[kScoreThreads / 32], span_hi[kScoreThreads / 32];
    const int b = static_cast<int>(blockIdx.x);
    const ScoreJob &job = jobs[find_job(jobs, count, b)];
    const int local = b - job.first_block;
    const int tile = local % job.column_tiles, segment = local / job.column_tiles;
    const int tid = static_cast<int>(threadIdx.x);
    const int s = tile * kScoreThreads + tid;
    const int lane = tid & 31, warp = tid >> 5;
    const int r0 = segment * job.segment_rows, r1 = min(job.height, r0 + job.segment_rows);
    {
        // Descaled rows touched by the segment (A_v rows list ascending j):
        // one segment row per thread, then a min / max reduction.
        int lo = job.rows, hi = -1;
        for (int r = r0 + tid; r < r1; r += kScoreThreads) {
            const std::uint32_t e0 = job.v.offsets[r], e1 = job.v.offsets[r + 1];
            if (e0 < e1) {
                lo = min(lo, job.v.indices[e0]);
                hi = max(hi, job.v.indices[e1 - 1]);
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
            hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
        }
        if (lane == 0) {
            span_lo[warp] = lo;
            span_hi[warp] = hi;
        }
    }
    __syncthreads();
    int j_lo = span_lo[0], j_hi = span_hi[0];
#pragma unroll
    for (int w = 1; w < kScoreThreads / 32; ++w) {
        j_lo = min(j_lo, span_lo[w]);
        j_hi = max(j_hi, span_hi[w]);
    }
    const int nj = j_hi - j_lo + 1;
    // The segment's A_v entries in shared memory when they fit; they are
    // read by every thread.
    const std::uint32_t v0 = job.v.offsets[r0], v1 = job.v.offsets[r1];
    const bool staged = v1 - v0 <= kScoreSegmentEntries && r1 - r0 <= kScoreMaxSegmentRows;
    if (staged) {
        for (std::uint32_t e = v0 + tid; e < v1; e += kScoreThreads)
            seg_e[e - v0] = make_float2(job.v.weights[e],
                                        __int_as_float((job.v.indices[e] - j_lo) * kScoreThreads * 4));
        for (int r = r0 + tid; r < r1; r += kScoreThreads) {
            const std::uint32_t e0 = job.v.offsets[r], e1 = job.v.offsets[r + 1];
            const int n = static_cast<int>(e1 - e0);
            const int first = n > 0 ? job.v.indices[e0] : j_lo;
            const bool consecutive = n > 0 && job.v.indices[e1 - 1] - first == n - 1;
            seg_r[r - r0] = make_int4(static_cast<int>(e0 - v0), n, (first - j_lo) * kScoreThreads * 4,
                                      consecutive ? 1 : 0);
        }
    }
    if (s < job.width) {
        // This column's A_h entries in registers (a tail beyond eight, rare,
        // reads them again from memory); the order of the sum is ascending.
        const std::uint32_t e0 = job.h.offsets[s], e1 = job.h.offsets[s + 1];
        const int ne = static_cast<int>(e1 - e0);
        constexpr int R = 8;
        float hw[R];
        int hc[R];
        const int c0 = ne > 0 ? job.h.indices[e0] : 0;
#pragma unroll
        for (int e = 0; e < R; ++e) {
            hw[e] = e < ne ? job.h.weights[e0 + e] : 0.0f;
            hc[e] = e < ne ? job.h.indices[e0 + e] - c0 : 0;
        }
        const bool run = ne > 0 && ne <= R && job.h.indices[e1 - 1] - c0 == ne - 1;
        const float *y = job.descaled + static_cast<std::int64_t>(j_lo) * job.descaled_stride + c0;
        const std::int64_t ys = job.descaled_stride;
        float *z = zt + tid;
        switch (ne) {
        case 0: for (int jj = 0; jj < nj; ++jj) z[jj * kScoreThreads] = 0.0f; break;
        case 1: row_pass<1>(z, y, ys, nj, run, hw, hc); break;
        case 2: row_pass<2>(z, y, ys, nj, run, hw, hc); break;
        case 3: row_pass<3>(z, y, ys, nj, run, hw, hc); break;
        case 4: row_pass<4>(z, y, ys, nj, run, hw, hc); break;
        case 5: row_pass<5>(z, y, ys, nj, run, hw, hc); break;
        case 6: row_pass<6>(z, y, ys, nj, run, hw, hc); break;
        case 7: row_pass<7>(z, y, ys, nj, run, hw, hc); break;
        default:
            for (int jj = 0; jj < nj; ++jj) {
                const float *yr = y + jj * ys;
                float acc = tap_sum<8>(yr, hw, hc);
                for (std::uint32_t e = e0 + R; e < e1; ++e) acc = fmaf(job.h.weights[e], yr[job.h.indices[e] - c0], acc);
                z[jj * kScoreThreads] = acc;
            }
            break;
        }
    }
    __syncthreads();
    const float *f = job.frame + s;
    const char *zb = reinterpret_cast<const char *>(zt + tid);
    const int row_blocks = (job.height + kScoreRowBlock - 1) / kScoreRowBlock;
    const int seg_blocks = job.segment_rows / kScoreRowBlock;
    const int rb_end = min(row_blocks, (segment + 1) * seg_blocks);
    int pending = 0;
    for (int rb = segment * seg_blocks; rb < rb_end; ++rb) {
        const int ra = rb * kScoreRowBlock, rz = min(job.height, ra + kScoreRowBlock);
        float sum = 0.0f;
        if (s < job.width) {
            // Two rows at a time, both frame samples loaded first (more
            // rows at once spill at this kernel's 64 registers).
            constexpr int kFetch = 2;
            for (int rf = ra; rf < rz; rf += kFetch) {
                const float *fr = f + static_cast<std::int64_t>(rf) * job.frame_stride;
                float fv[kFetch];
#pragma unroll
                for (int k = 0; k < kFetch; ++k)
                    fv[k] = rf + k < rz ? __ldg(fr + static_cast<std::int64_t>(k) * job.frame_stride) : 0.0f;
#pragma unroll
                for (int k = 0; k < kFetch; ++k) {
                    const int r = rf + k;
                    if (r >= rz) continue;
                    float acc = 0.0f;
                    if (staged) {
                        const int4 h = seg_r[r - r0];
                        const float2 *we = seg_e + h.x;
                        const char *zr = zb + h.z;
                        if (h.w) {
                            switch (h.y) {
                            case 1: acc = col_run<1>(we, zr); break;
                            case 2: acc = col_run<2>(we, zr); break;
                            case 3: acc = col_run<3>(we, zr); break;
                            case 4: acc = col_run<4>(we, zr); break;
                            case 5: acc = col_run<5>(we, zr); break;
                            case 6: acc = col_run<6>(we, zr); break;
                            case 7: acc = col_run<7>(we, zr); break;
                            case 8: acc = col_run<8>(we, zr); break;
                            default:
                                for (int e = 0; e < h.y; ++e)
                                    acc = fmaf(we[e].x, *reinterpret_cast<const float *>(zr + e * kScoreThreads * 4), acc);
                                break;
                            }
                        } else {
                            for (int e = 0; e < h.y; ++e)
                                acc = fmaf(we[e].x, *reinterpret_cast<const float *>(zb + __float_as_int(we[e].y)), acc);
                        }
                    } else {
                        const std::uint32_t e0 = job.v.offsets[r], e1 = job.v.offsets[r + 1];
                        for (std::uint32_t e = e0; e < e1; ++e)
                            acc = fmaf(job.v.weights[e], zt[(job.v.indices[e] - j_lo) * kScoreThreads + tid], acc);
                    }
                    sum += fabsf(acc - fv[k]);
                }
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) sum += __shfl_down_sync(0xffffffffu, sum, o);
        if (lane == 0) warp_sums[pending * kWarps + warp] = sum;
        // The pending blocks' sums, one thread a block, after the last
        // block of the segment (or when the buffer is full).
        if (++pending == kPendingBlocks || rb + 1 == rb_end) {
            __syncthreads();
            if (tid < pending) {
                float total = 0.0f;
                for (int w = 0; w < kWarps; ++w) total += warp_sums[tid * kWarps + w];
                job.partials[static_cast<std::int64_t>(rb + 1 - pending + tid) * job.column_tiles + tile] = total;
            }
            __syncthreads();
            pending = 0;
        }
    }
}

__global__ void __launch_bounds__(kScoreThreads)
score_finalize_kernel(const ScoreJob *__restrict__ jobs) {
    __shared__ double sums[kScoreThreads];
    const ScoreJob &job = jobs[blockIdx.x];
    const int n = job.column_tiles * ((job.height + kScoreRowBlock - 1) / kScoreRowBlock);
    double acc = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) acc += static_cast<double>(job.partials[i]);
    sums[threadIdx.x] = acc;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (static_cast<int>(threadIdx.x) < w) sums[threadIdx.x] += sums[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0)
        *job.score = static_cast<float>(sums[0] / (static_cast<double>(job.width) * job.height));
}

__global__ void __launch_bounds__(kScoreThreads)
fused_score_finalize_kernel(const dev::ScoreEpilogue *__restrict__ epilogues) {
    __shared__ double sums[kScoreThreads];
    const dev::ScoreEpilogue &ep = epilogues[blockIdx.x];
    double acc = 0.0;
    for (int i = threadIdx.x; i < ep.tiles; i += blockDim.x) acc += ep.partials[i];
    sums[threadIdx.x] = acc;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (static_cast<int>(threadIdx.x) < w) sums[threadIdx.x] += sums[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0)
        *ep.score = static_cast<float>(sums[0] / (static_cast<double>(ep.width) * ep.height));
}

} // namespace

int launch_fused_score_finalize(const dev::ScoreEpilogue *epilogues, int count, void *stream) {
    if (count <= 0) return 0;
    fused_score_finalize_kernel<<<count, kScoreThreads, 0, static_cast<cudaStream_t>(stream)>>>(epilogues);
    return static_cast<int>(cudaGetLastError());
}

int launch_score_tiles(const dev::ScoreJob *jobs, int count, int blocks, int max_span_rows, void *stream) {
    if (blocks <= 0) return 0;
    const int smem = max_span_rows * kScoreThreads * static_cast<int>(sizeof(float));
    // The kernel's static shared memory counts against the default 48 KiB
    // too, so the dynamic limit is raised for any size not configured yet.
    static SmemLimit limit;
    if (const cudaError_t e = limit.ensure(score_tiles_kernel, smem); e != cudaSuccess) return static_cast<int>(e);
    score_tiles_kernel<<<blocks, kScoreThreads, smem, static_cast<cudaStream_t>(stream)>>>(jobs, count);
    return static_cast<int>(cudaGetLastError());
}

int launch_score_finalize(const dev::ScoreJob *jobs, int count, void *stream) {
    if (count <= 0) return 0;
    score_finalize_kernel<<<count, kScoreThreads, 0, static_cast<cudaStream_t>(stream)>>>(jobs);
    return static_cast<int>(cudaGetLastError());
}

} // namespace dsmvc_gb
