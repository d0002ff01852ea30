// Host<->device plane copies.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>

namespace dsmvc_gb {

// cudaMemcpy2DAsync's arguments; a plane whose rows are contiguous on both
// sides goes as one linear copy (pitched copies move row by row, far below
// the link's bandwidth for rows of a few KiB).
inline cudaError_t copy_plane(void *dst, std::size_t dpitch, const void *src, std::size_t spitch,
                              std::size_t width, std::size_t rows, cudaMemcpyKind kind, cudaStream_t stream) {
    if (dpitch == width && spitch == width) return cudaMemcpyAsync(dst, src, width * rows, kind, stream);
    return cudaMemcpy2DAsync(dst, dpitch, src, spitch, width, rows, kind, stream);
}

} // namespace dsmvc_gb
