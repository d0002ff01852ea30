// Two-pass transposing kernels for half-bandwidth 11 (see tsolve_impl.cuh);
// one translation unit per half-bandwidth.
#include "tsolve_impl.cuh"

namespace dsmvc_gb {

int launch_tsolve_hb11(const dev::StreamJob *jobs, int count, int blocks, int threads, int window,
                       dev::Sample in, dev::Sample out, int record_floats, void *stream) {
    auto s = static_cast<cudaStream_t>(stream);
    if (window == 8) return xlaunch_k<11, 8>(jobs, count, blocks, threads, in, out, record_floats, s);
    return xlaunch_k<11, 0>(jobs, count, blocks, threads, in, out, record_floats, s);
}

} // namespace dsmvc_gb
