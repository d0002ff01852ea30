// Candidate scoring kernels (score.cuh).
#include "score.cuh"

#include <cuda_runtime.h>

namespace dsmvc_gb {
namespace {

using dev::ScoreJob;

__device__ __forceinline__ int find_job(const ScoreJob *jobs, int count, int block, bool rows) {
    int lo = 0, hi = count - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        const int first = rows ? jobs[mid].first_block_rows : jobs[mid].first_block_cols;
        if (first <= block) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// Z[j][s] = sum_e A_h[s, e] * Y[j][e] for one descaled row j.
__global__ void __launch_bounds__(kScoreThreads)
upscale_rows_kernel(const ScoreJob *__restrict__ jobs, int count) {
    extern __shared__ float row[];
    const int b = static_cast<int>(blockIdx.x);
    const ScoreJob &job = jobs[find_job(jobs, count, b, true)];
    const int j = b - job.first_block_rows;
    const float *y = job.descaled + static_cast<std::int64_t>(j) * job.descaled_stride;
    for (int c = threadIdx.x; c < job.cols; c += blockDim.x) row[c] = y[c];
    __syncthreads();
    float *z = job.upscaled_rows + static_cast<std::int64_t>(j) * job.upscaled_stride;
    for (int s = threadIdx.x; s < job.width; s += blockDim.x) {
        const std::uint32_t e0 = job.h.offsets[s], e1 = job.h.offsets[s + 1];
        float acc = 0.0f;
        for (std::uint32_t e = e0; e < e1; ++e) acc = fmaf(job.h.weights[e], row[job.h.indices[e]], acc);
        z[s] = acc;
    }
}

// For one column tile and one segment of source rows: the upscaled sample
// sum_e A_v[r, e] * Z[e][s] against frame[r][s].  Absolute errors are summed
// per block of kScoreRowBlock rows (one partial per column tile and row
// block, whatever the segment length), so the partial sums -- and the
// score -- do not depend on the segment a launch uses.
__global__ void __launch_bounds__(kScoreThreads)
upscale_columns_l1_kernel(const ScoreJob *__restrict__ jobs, int count) {
    __shared__ float warp_sums[kScoreThreads / 32];
    const int b = static_cast<int>(blockIdx.x);
    const ScoreJob &job = jobs[find_job(jobs, count, b, false)];
    const int local = b - job.first_block_cols;
    const int tile = local % job.column_tiles, segment = local / job.column_tiles;
    const int s = tile * static_cast<int>(blockDim.x) + static_cast<int>(threadIdx.x);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int row_blocks = (job.height + kScoreRowBlock - 1) / kScoreRowBlock;
    const int seg_blocks = job.segment_rows / kScoreRowBlock;
    const float *z = job.upscaled_rows + s;
    const float *f = job.frame + s;
    for (int rb = segment * seg_blocks; rb < min(row_blocks, (segment + 1) * seg_blocks); ++rb) {
        const int r0 = rb * kScoreRowBlock, r1 = min(job.height, r0 + kScoreRowBlock);
        float sum = 0.0f;
        if (s < job.width) {
            for (int r = r0; r < r1; ++r) {
                const std::uint32_t e0 = job.v.offsets[r], e1 = job.v.offsets[r + 1];
                float acc = 0.0f;
                for (std::uint32_t e = e0; e < e1; ++e)
                    acc = fmaf(job.v.weights[e], z[static_cast<std::int64_t>(job.v.indices[e]) * job.upscaled_stride],
                               acc);
                sum += fabsf(acc - f[static_cast<std::int64_t>(r) * job.frame_stride]);
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) sum += __shfl_down_sync(0xffffffffu, sum, o);
        if (lane == 0) warp_sums[warp] = sum;
        __syncthreads();
        if (threadIdx.x == 0) {
            float total = 0.0f;
            for (int w = 0; w < static_cast<int>(blockDim.x) / 32; ++w) total += warp_sums[w];
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

int launch_upscale_rows(const dev::ScoreJob *jobs, int count, int blocks, int max_cols, void *stream) {
    if (blocks <= 0) return 0;
    const int smem = max_cols * static_cast<int>(sizeof(float));
    static int configured = 0;
    if (smem > 48 * 1024 && smem > configured) {
        const cudaError_t e = cudaFuncSetAttribute(upscale_rows_kernel,
                                                   cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e != cudaSuccess) return static_cast<int>(e);
        configured = smem;
    }
    upscale_rows_kernel<<<blocks, kScoreThreads, smem, static_cast<cudaStream_t>(stream)>>>(jobs, count);
    return static_cast<int>(cudaGetLastError());
}

int launch_upscale_columns_l1(const dev::ScoreJob *jobs, int count, int blocks, void *stream) {
    if (blocks <= 0) return 0;
    upscale_columns_l1_kernel<<<blocks, kScoreThreads, 0, static_cast<cudaStream_t>(stream)>>>(jobs, count);
    return static_cast<int>(cudaGetLastError());
}

int launch_score_finalize(const dev::ScoreJob *jobs, int count, float *scores, void *stream) {
    if (count <= 0) return 0;
    score_finalize_kernel<<<count, kScoreThreads, 0, static_cast<cudaStream_t>(stream)>>>(jobs, scores);
    return static_cast<int>(cudaGetLastError());
}

} // namespace dsmvc_gb
