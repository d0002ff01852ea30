// Dynamic shared-memory limits of kernels launched from many host threads.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <mutex>

namespace dsmvc_gb {

// The dynamic shared-memory limit configured so far for one kernel, per
// device.  Host-call slots launch the same kernel from several threads, and
// the attribute belongs to the kernel on the current device, so the limit
// only grows, under a lock, and a launch never follows a lowered limit.
class SmemLimit {
public:
    // Raises `kernel`'s limit on the current device to at least `bytes`.
    template <class Kernel> cudaError_t ensure(Kernel kernel, int bytes) {
        int device = 0;
        cudaError_t e = cudaGetDevice(&device);
        if (e != cudaSuccess) return e;
        if (device < 0 || device >= kDevices) return cudaErrorInvalidDevice;
        if (bytes <= have_[device].load(std::memory_order_acquire)) return cudaSuccess;
        std::lock_guard<std::mutex> lock(mutex_);
        if (bytes <= have_[device].load(std::memory_order_relaxed)) return cudaSuccess;
        e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
        if (e == cudaSuccess) have_[device].store(bytes, std::memory_order_release);
        return e;
    }

private:
    static constexpr int kDevices = 64;
    std::mutex mutex_;
    std::atomic<int> have_[kDevices] = {};
};

} // namespace dsmvc_gb
