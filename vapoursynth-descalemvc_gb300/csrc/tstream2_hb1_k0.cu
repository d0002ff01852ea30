// Paired transposing streaming kernels for half-bandwidth 1, other windows
// (see tstream2_impl.cuh); one translation unit per half-bandwidth and
// window variant keeps each compile short.
#include "tstream2_impl.cuh"

namespace dsmvc_gb {

int launch_tstream2_hb1_k0(const dev::StreamJob *jobs, int count, int blocks, int threads, dev::Sample in,
                          dev::Sample out, int record_floats, void *stream) {
    return plaunch_k<1, 0>(jobs, count, blocks, threads, in, out, record_floats,
                              static_cast<cudaStream_t>(stream));
}

} // namespace dsmvc_gb
