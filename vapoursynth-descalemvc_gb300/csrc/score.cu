// Candidate scoring kernels (score.cuh).
#include "score.cuh"

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

// Fused re-upscale and error sum of one column tile x one row segment of a
// candidate: the row-pass values Z[j][s] = sum_c A_h[s, c] Y[j][c] of the
// rows j the segment needs are computed into shared memory, then each
// source row r of the segment is sum_j A_v[r, j] Z[j][s], compared with the
// frame.  Errors are summed per block of kScoreRowBlock rows.
__global__ void __launch_bounds__(kScoreThreads)
score_tiles_kernel(const ScoreJob *__restrict__ jobs, int count) {
    extern __shared__ float zt[];                  // [rows of the segment's span][kScoreThreads]
    __shared__ float warp_sums[kScoreThreads / 32];
    __shared__ float seg_w[kScoreSegmentEntries];
    __shared__ int seg_j[kScoreSegmentEntries];
    __shared__ int span[2];
    const int b = static_cast<int>(blockIdx.x);
    const ScoreJob &job = jobs[find_job(jobs, count, b)];
    const int local = b - job.first_block;
    const int tile = local % job.column_tiles, segment = local / job.column_tiles;
    const int tid = static_cast<int>(threadIdx.x);
    const int s = tile * kScoreThreads + tid;
    const int lane = tid & 31, warp = tid >> 5;
    const int r0 = segment * job.segment_rows, r1 = min(job.height, r0 + job.segment_rows);
    if (tid == 0) {
        // Descaled rows touched by the segment (A_v rows list ascending j).
        int lo = job.rows, hi = -1;
        for (int r = r0; r < r1; ++r) {
            const std::uint32_t e0 = job.v.offsets[r], e1 = job.v.offsets[r + 1];
            if (e0 < e1) {
                lo = min(lo, job.v.indices[e0]);
                hi = max(hi, job.v.indices[e1 - 1]);
            }
        }
        span[0] = lo;
        span[1] = hi;
    }
    __syncthreads();
    const int j_lo = span[0], nj = span[1] - span[0] + 1;
    // The segment's A_v entries (weights and staged-row offsets) in shared
    // memory when they fit; they are read by every thread.
    const std::uint32_t v0 = job.v.offsets[r0], v1 = job.v.offsets[r1];
    const bool staged = v1 - v0 <= kScoreSegmentEntries;
    if (staged) {
        for (std::uint32_t e = v0 + tid; e < v1; e += kScoreThreads) {
            seg_w[e - v0] = job.v.weights[e];
            seg_j[e - v0] = (job.v.indices[e] - j_lo) * kScoreThreads;
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
#pragma unroll
        for (int e = 0; e < R; ++e) {
            hw[e] = e < ne ? job.h.weights[e0 + e] : 0.0f;
            hc[e] = e < ne ? job.h.indices[e0 + e] : 0;
        }
        for (int jj = 0; jj < nj; ++jj) {
            const float *y = job.descaled + static_cast<std::int64_t>(j_lo + jj) * job.descaled_stride;
            float acc = 0.0f;
#pragma unroll
            for (int e = 0; e < R; ++e)
                if (e < ne) acc = fmaf(hw[e], y[hc[e]], acc);
            for (std::uint32_t e = e0 + R; e < e1; ++e) acc = fmaf(job.h.weights[e], y[job.h.indices[e]], acc);
            zt[jj * kScoreThreads + tid] = acc;
        }
    }
    __syncthreads();
    const float *f = job.frame + s;
    const int row_blocks = (job.height + kScoreRowBlock - 1) / kScoreRowBlock;
    const int seg_blocks = job.segment_rows / kScoreRowBlock;
    for (int rb = segment * seg_blocks; rb < min(row_blocks, (segment + 1) * seg_blocks); ++rb) {
        const int ra = rb * kScoreRowBlock, rz = min(job.height, ra + kScoreRowBlock);
        float sum = 0.0f;
        if (s < job.width) {
            for (int r = ra; r < rz; ++r) {
                const std::uint32_t e0 = job.v.offsets[r], e1 = job.v.offsets[r + 1];
                float acc = 0.0f;
                if (staged) {
                    for (std::uint32_t e = e0 - v0; e < e1 - v0; ++e) acc = fmaf(seg_w[e], zt[seg_j[e] + tid], acc);
                } else {
                    for (std::uint32_t e = e0; e < e1; ++e)
                        acc = fmaf(job.v.weights[e], zt[(job.v.indices[e] - j_lo) * kScoreThreads + tid], acc);
                }
                sum += fabsf(acc - f[static_cast<std::int64_t>(r) * job.frame_stride]);
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) sum += __shfl_down_sync(0xffffffffu, sum, o);
        if (lane == 0) warp_sums[warp] = sum;
        __syncthreads();
        if (tid == 0) {
            float total = 0.0f;
            for (int w = 0; w < kScoreThreads / 32; ++w) total += warp_sums[w];
            job.partials[static_cast<std::int64_t>(rb) * job.column_tiles + tile] = total;
        }
        __syncthreads();
    }
}

__global__ void __launch_bounds__(kScoreThreads)
score_finalize_kernel(const ScoreJob *__restrict__ jobs, float *scores) {
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
        scores[blockIdx.x] = static_cast<float>(sums[0] / (static_cast<double>(job.width) * job.height));
}

} // namespace

int launch_score_tiles(const dev::ScoreJob *jobs, int count, int blocks, int max_span_rows, void *stream) {
    if (blocks <= 0) return 0;
    const int smem = max_span_rows * kScoreThreads * static_cast<int>(sizeof(float));
    // The kernel's static shared memory counts against the default 48 KiB
    // too, so the dynamic limit is raised for any size not configured yet.
    static int configured = 0;
    if (smem > configured) {
        const cudaError_t e = cudaFuncSetAttribute(score_tiles_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                   smem);
        if (e != cudaSuccess) return static_cast<int>(e);
        configured = smem;
    }
    score_tiles_kernel<<<blocks, kScoreThreads, smem, static_cast<cudaStream_t>(stream)>>>(jobs, count);
    return static_cast<int>(cudaGetLastError());
}

int launch_score_finalize(const dev::ScoreJob *jobs, int count, float *scores, void *stream) {
    if (count <= 0) return 0;
    score_finalize_kernel<<<count, kScoreThreads, 0, static_cast<cudaStream_t>(stream)>>>(jobs, scores);
    return static_cast<int>(cudaGetLastError());
}

} // namespace dsmvc_gb
