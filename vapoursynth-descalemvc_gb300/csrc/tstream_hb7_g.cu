// Transposing streaming kernels with grouped records for half-bandwidth 7
// (see tstream_impl.cuh); one translation unit per half-bandwidth.
#include "tstream_impl.cuh"

namespace dsmvc_gb {

int launch_tstream_g_hb7(const dev::StreamJob *jobs, int count, int blocks, int threads, int window,
                          dev::Sample in, dev::Sample out, int record_floats, void *stream) {
    return tlaunch_hb_grouped<7>(jobs, count, blocks, threads, window, in, out, record_floats,
                                  static_cast<cudaStream_t>(stream));
}

} // namespace dsmvc_gb
