// Streaming axis kernels for half-bandwidth 7 (see stream_impl.cuh); one
// translation unit per half-bandwidth keeps the build parallel.
#include "stream_impl.cuh"

namespace dsmvc_gb {

int launch_stream_hb7(const dev::StreamJob *jobs, int count, int blocks, bool contiguous,
                        dev::Sample in, dev::Sample out, int record_floats, void *stream) {
    return launch_hb<7, kStreamChunk>(jobs, count, blocks, contiguous, in, out, record_floats,
                                       static_cast<cudaStream_t>(stream));
}

} // namespace dsmvc_gb
