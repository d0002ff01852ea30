// Measured device peaks (peak.cu).
#pragma once

namespace dsmvc_gb {

// FP64 TFLOP/s (two per FMA) of `device`; returns a cudaError_t as int.
int measure_fp64_peak(int device, double *tflops);

} // namespace dsmvc_gb
