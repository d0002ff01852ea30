// Float64 two-pass transposing kernels for half-bandwidth 1 (see
// tsolve64_impl.cuh); one translation unit per half-bandwidth.
#include "tsolve64_impl.cuh"

namespace dsmvc_gb {

int launch_tsolve64_hb1(const dev::StreamJob *jobs, int count, int blocks, int threads, dev::Sample in,
                         dev::Sample out, int record_floats, bool fused, std::uint32_t *status, void *stream) {
    return x64launch_hb<1>(jobs, count, blocks, threads, in, out, record_floats, fused, status,
                            static_cast<cudaStream_t>(stream));
}

} // namespace dsmvc_gb
