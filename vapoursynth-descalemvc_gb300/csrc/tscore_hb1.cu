// Columns passes with fused candidate scoring for half-bandwidth 1
// (tscore_impl.cuh); one translation unit per half-bandwidth.
#include "tscore_impl.cuh"

namespace dsmvc_gb {

int launch_tscore_hb1(const dev::StreamJob *jobs, int count, int blocks, int window, int record_floats,
                       void *stream) {
    return tscore_launch_hb<1>(jobs, count, blocks, window, record_floats, static_cast<cudaStream_t>(stream));
}

} // namespace dsmvc_gb
