// Paired transposing streaming kernels for half-bandwidth 5, window 8
// (see tstream2_impl.cuh); one translation unit per half-bandwidth and
// window variant keeps each compile short.
#include "tstream2_impl.cuh"

namespace dsmvc_gb {

int launch_tstream2_hb5_k8(const dev::StreamJob *jobs, int count, int blocks, int threads, dev::Sample in,
                          dev::Sample out, int record_floats, void *stream) {
    return plaunch_k<5, 8>(jobs, count, blocks, threads, in, out, record_floats,
                              static_cast<cudaStream_t>(stream));
}

} // namespace dsmvc_gb
