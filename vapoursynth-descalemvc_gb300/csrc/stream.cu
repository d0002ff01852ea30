// Dispatch of the streaming axis kernels by half-bandwidth.
#include "stream.cuh"

#include <cuda_runtime.h>

namespace dsmvc_gb {

int launch_stream_hb1(const dev::StreamJob *, int, int, bool, dev::Sample, dev::Sample, int, void *);
int launch_stream_hb3(const dev::StreamJob *, int, int, bool, dev::Sample, dev::Sample, int, void *);
int launch_stream_hb5(const dev::StreamJob *, int, int, bool, dev::Sample, dev::Sample, int, void *);
int launch_stream_hb7(const dev::StreamJob *, int, int, bool, dev::Sample, dev::Sample, int, void *);

int stream_threads() { return 128; }

bool stream_supports(int half_bandwidth) {
    return half_bandwidth == 1 || half_bandwidth == 3 || half_bandwidth == 5 || half_bandwidth == 7;
}

int launch_stream(const dev::StreamJob *jobs, int job_count, int total_blocks, int half_bandwidth,
                  int chunk, bool contiguous, dev::Sample in, dev::Sample out, int record_floats,
                  void *stream) {
    if (chunk != kStreamChunk) return static_cast<int>(cudaErrorInvalidValue);
    switch (half_bandwidth) {
    case 1: return launch_stream_hb1(jobs, job_count, total_blocks, contiguous, in, out, record_floats, stream);
    case 3: return launch_stream_hb3(jobs, job_count, total_blocks, contiguous, in, out, record_floats, stream);
    case 5: return launch_stream_hb5(jobs, job_count, total_blocks, contiguous, in, out, record_floats, stream);
    case 7: return launch_stream_hb7(jobs, job_count, total_blocks, contiguous, in, out, record_floats, stream);
    default: return static_cast<int>(cudaErrorInvalidValue);
    }
}

} // namespace dsmvc_gb

namespace dsmvc_gb {

int launch_tstream_hb1(const dev::StreamJob *, int, int, int, int, dev::Sample, dev::Sample, int, void *);
int launch_tstream_hb3(const dev::StreamJob *, int, int, int, int, dev::Sample, dev::Sample, int, void *);
int launch_tstream_hb5(const dev::StreamJob *, int, int, int, int, dev::Sample, dev::Sample, int, void *);
int launch_tstream_hb7(const dev::StreamJob *, int, int, int, int, dev::Sample, dev::Sample, int, void *);

int launch_tstream2_hb1_k0(const dev::StreamJob *, int, int, int, dev::Sample, dev::Sample, int, void *);
int launch_tstream2_hb1_k8(const dev::StreamJob *, int, int, int, dev::Sample, dev::Sample, int, void *);
int launch_tstream2_hb3_k0(const dev::StreamJob *, int, int, int, dev::Sample, dev::Sample, int, void *);
int launch_tstream2_hb3_k8(const dev::StreamJob *, int, int, int, dev::Sample, dev::Sample, int, void *);
int launch_tstream2_hb5_k0(const dev::StreamJob *, int, int, int, dev::Sample, dev::Sample, int, void *);
int launch_tstream2_hb5_k8(const dev::StreamJob *, int, int, int, dev::Sample, dev::Sample, int, void *);
int launch_tstream2_hb7_k0(const dev::StreamJob *, int, int, int, dev::Sample, dev::Sample, int, void *);
int launch_tstream2_hb7_k8(const dev::StreamJob *, int, int, int, dev::Sample, dev::Sample, int, void *);

int launch_tstream2(const dev::StreamJob *jobs, int job_count, int total_blocks, int threads, int half_bandwidth,
                    int window, dev::Sample in, dev::Sample out, int record_floats, void *stream) {
    const bool k8 = window == 8;
#define DSMVC_PAIRED(H)                                                                                        \
    case H:                                                                                                    \
        return k8 ? launch_tstream2_hb##H##_k8(jobs, job_count, total_blocks, threads, in, out, record_floats, \
                                               stream)                                                         \
                  : launch_tstream2_hb##H##_k0(jobs, job_count, total_blocks, threads, in, out, record_floats, \
                                               stream);
    switch (half_bandwidth) {
        DSMVC_PAIRED(1)
        DSMVC_PAIRED(3)
        DSMVC_PAIRED(5)
        DSMVC_PAIRED(7)
    default: return static_cast<int>(cudaErrorInvalidValue);
    }
#undef DSMVC_PAIRED
}

int launch_tsolve_hb1(const dev::StreamJob *, int, int, int, int, dev::Sample, dev::Sample, int, void *);
int launch_tsolve_hb3(const dev::StreamJob *, int, int, int, int, dev::Sample, dev::Sample, int, void *);
int launch_tsolve_hb5(const dev::StreamJob *, int, int, int, int, dev::Sample, dev::Sample, int, void *);
int launch_tsolve_hb7(const dev::StreamJob *, int, int, int, int, dev::Sample, dev::Sample, int, void *);
int launch_tsolve_hb9(const dev::StreamJob *, int, int, int, int, dev::Sample, dev::Sample, int, void *);
int launch_tsolve_hb11(const dev::StreamJob *, int, int, int, int, dev::Sample, dev::Sample, int, void *);

int launch_tsolve64_hb1(const dev::StreamJob *, int, int, int, dev::Sample, dev::Sample, int, bool, std::uint32_t *, void *);
int launch_tsolve64_hb3(const dev::StreamJob *, int, int, int, dev::Sample, dev::Sample, int, bool, std::uint32_t *, void *);
int launch_tsolve64_hb5(const dev::StreamJob *, int, int, int, dev::Sample, dev::Sample, int, bool, std::uint32_t *, void *);
int launch_tsolve64_hb7(const dev::StreamJob *, int, int, int, dev::Sample, dev::Sample, int, bool, std::uint32_t *, void *);
int launch_tsolve64_hb9(const dev::StreamJob *, int, int, int, dev::Sample, dev::Sample, int, bool, std::uint32_t *, void *);
int launch_tsolve64_hb11(const dev::StreamJob *, int, int, int, dev::Sample, dev::Sample, int, bool, std::uint32_t *, void *);

int launch_tsolve64(const dev::StreamJob *jobs, int job_count, int total_blocks, int threads, int half_bandwidth,
                    dev::Sample in, dev::Sample out, int record_floats, bool fused, std::uint32_t *status,
                    void *stream) {
    switch (half_bandwidth) {
    case 1: return launch_tsolve64_hb1(jobs, job_count, total_blocks, threads, in, out, record_floats, fused, status, stream);
    case 3: return launch_tsolve64_hb3(jobs, job_count, total_blocks, threads, in, out, record_floats, fused, status, stream);
    case 5: return launch_tsolve64_hb5(jobs, job_count, total_blocks, threads, in, out, record_floats, fused, status, stream);
    case 7: return launch_tsolve64_hb7(jobs, job_count, total_blocks, threads, in, out, record_floats, fused, status, stream);
    case 9: return launch_tsolve64_hb9(jobs, job_count, total_blocks, threads, in, out, record_floats, fused, status, stream);
    case 11: return launch_tsolve64_hb11(jobs, job_count, total_blocks, threads, in, out, record_floats, fused, status, stream);
    default: return static_cast<int>(cudaErrorInvalidValue);
    }
}

bool tsolve_supports(int half_bandwidth) {
    return half_bandwidth >= 1 && half_bandwidth <= 11 && half_bandwidth % 2 == 1;
}

int launch_tsolve(const dev::StreamJob *jobs, int job_count, int total_blocks, int threads, int half_bandwidth,
                  int window, dev::Sample in, dev::Sample out, int record_floats, void *stream) {
    switch (half_bandwidth) {
    case 1: return launch_tsolve_hb1(jobs, job_count, total_blocks, threads, window, in, out, record_floats, stream);
    case 3: return launch_tsolve_hb3(jobs, job_count, total_blocks, threads, window, in, out, record_floats, stream);
    case 5: return launch_tsolve_hb5(jobs, job_count, total_blocks, threads, window, in, out, record_floats, stream);
    case 7: return launch_tsolve_hb7(jobs, job_count, total_blocks, threads, window, in, out, record_floats, stream);
    case 9: return launch_tsolve_hb9(jobs, job_count, total_blocks, threads, window, in, out, record_floats, stream);
    case 11: return launch_tsolve_hb11(jobs, job_count, total_blocks, threads, window, in, out, record_floats, stream);
    default: return static_cast<int>(cudaErrorInvalidValue);
    }
}

int launch_tstream_g_hb1(const dev::StreamJob *, int, int, int, int, dev::Sample, dev::Sample, int, void *);
int launch_tstream_g_hb3(const dev::StreamJob *, int, int, int, int, dev::Sample, dev::Sample, int, void *);
int launch_tstream_g_hb5(const dev::StreamJob *, int, int, int, int, dev::Sample, dev::Sample, int, void *);
int launch_tstream_g_hb7(const dev::StreamJob *, int, int, int, int, dev::Sample, dev::Sample, int, void *);

int launch_tstream(const dev::StreamJob *jobs, int job_count, int total_blocks, int threads, int half_bandwidth,
                   int window, dev::Sample in, dev::Sample out, int record_floats, void *stream) {
    if (window > 8) {
        switch (half_bandwidth) {
        case 1: return launch_tstream_g_hb1(jobs, job_count, total_blocks, threads, window, in, out, record_floats, stream);
        case 3: return launch_tstream_g_hb3(jobs, job_count, total_blocks, threads, window, in, out, record_floats, stream);
        case 5: return launch_tstream_g_hb5(jobs, job_count, total_blocks, threads, window, in, out, record_floats, stream);
        case 7: return launch_tstream_g_hb7(jobs, job_count, total_blocks, threads, window, in, out, record_floats, stream);
        default: return static_cast<int>(cudaErrorInvalidValue);
        }
    }
    switch (half_bandwidth) {
    case 1: return launch_tstream_hb1(jobs, job_count, total_blocks, threads, window, in, out, record_floats, stream);
    case 3: return launch_tstream_hb3(jobs, job_count, total_blocks, threads, window, in, out, record_floats, stream);
    case 5: return launch_tstream_hb5(jobs, job_count, total_blocks, threads, window, in, out, record_floats, stream);
    case 7: return launch_tstream_hb7(jobs, job_count, total_blocks, threads, window, in, out, record_floats, stream);
    default: return static_cast<int>(cudaErrorInvalidValue);
    }
}

int launch_tscore_hb1(const dev::StreamJob *, int, int, int, int, void *);
int launch_tscore_hb3(const dev::StreamJob *, int, int, int, int, void *);
int launch_tscore_hb5(const dev::StreamJob *, int, int, int, int, void *);
int launch_tscore_hb7(const dev::StreamJob *, int, int, int, int, void *);

int launch_tscore(const dev::StreamJob *jobs, int job_count, int total_blocks, int half_bandwidth, int window,
                  int record_floats, void *stream) {
    switch (half_bandwidth) {
    case 1: return launch_tscore_hb1(jobs, job_count, total_blocks, window, record_floats, stream);
    case 3: return launch_tscore_hb3(jobs, job_count, total_blocks, window, record_floats, stream);
    case 5: return launch_tscore_hb5(jobs, job_count, total_blocks, window, record_floats, stream);
    case 7: return launch_tscore_hb7(jobs, job_count, total_blocks, window, record_floats, stream);
    default: return static_cast<int>(cudaErrorInvalidValue);
    }
}

} // namespace dsmvc_gb
