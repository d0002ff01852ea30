// Measured FP64 FMA throughput of the device: the denominator of the
// Float64 route's FLOP roofline (the device's nominal FP64 rate is far below
// its Float32 rate, so it is measured rather than assumed).
#include "peak.hpp"

#include <cuda_runtime.h>

namespace dsmvc_gb {
namespace {

// Eight independent FMA chains per thread; one store per thread into an
// array of grid x block doubles.
__global__ void dfma_chains(double *out, int iterations, double a, double b) {
    double x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6,
           x7 = x0 + 7;
    for (int i = 0; i < iterations; ++i) {
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
            x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
        }
    }
    out[static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

} // namespace

// FP64 TFLOP/s (2 per FMA) of the best of three timed launches.
int measure_fp64_peak(int device, double *tflops) {
    int previous = -1;
    cudaGetDevice(&previous);
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return static_cast<int>(e);
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const int blocks = sms * 8, threads = 256, iterations = 256;
    double *out = nullptr;
    cudaEvent_t start = nullptr, stop = nullptr;
    double best = 0.0;
    e = cudaMalloc(&out, static_cast<size_t>(blocks) * threads * sizeof(double));
    if (e == cudaSuccess) e = cudaEventCreate(&start);
    if (e == cudaSuccess) e = cudaEventCreate(&stop);
    for (int rep = 0; rep < 4 && e == cudaSuccess; ++rep) {
        cudaEventRecord(start);
        dfma_chains<<<blocks, threads>>>(out, iterations, 0.999, 0.001);
        cudaEventRecord(stop);
        e = cudaEventSynchronize(stop);
        float ms = 0.0F;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, start, stop);
        const double fmas = static_cast<double>(blocks) * threads * iterations * 64.0;
        if (e == cudaSuccess && rep > 0 && ms > 0.0F) best = best > 2.0 * fmas / ms / 1e9 ? best : 2.0 * fmas / ms / 1e9;
    }
    if (start) cudaEventDestroy(start);
    if (stop) cudaEventDestroy(stop);
    if (out) cudaFree(out);
    if (previous >= 0) cudaSetDevice(previous);
    *tflops = best;
    return static_cast<int>(e);
}

} // namespace dsmvc_gb
