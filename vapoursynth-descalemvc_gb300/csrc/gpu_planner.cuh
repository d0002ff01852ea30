// Device planner: the normal-matrix band, its banded LDL^T factor, the
// three-stage reciprocal condition estimate and the Float32 solve arrays of
// many axis plans at once, on the GPU, bit-identical to the host planner
// (planner.cpp, in the reference planner's operation order,
// src/axis_plan.cpp:628-967).  The host keeps the O(n * taps) part -- the
// sampling geometry and kernel weights (its libm sin/cos), the coalesced
// descale matrix and its transpose -- and hands the A^T CSR over.
#pragma once

#include <cstddef>
#include <cstdint>

namespace dsmvc_gb {

// One plan of a device planning batch: sizes and offsets into the batch's
// packed arrays (elements, not bytes).
struct PlannerJob {
    std::int32_t n = 0;              // destination size
    std::int32_t hb = 0;             // half-bandwidth
    std::int32_t mode = 0;           // F64Mode
    std::int32_t pad = 0;
    std::int64_t offsets_at = 0;     // A^T CSR offsets (n + 1, relative to entries_at)
    std::int64_t entries_at = 0;     // A^T CSR indices and Float64 weights
    std::int64_t bands_at = 0;       // normal bands and LDL^T factor, (hb + 1) * n doubles each
    std::int64_t factors_at = 0;     // lower_ld and upper_l, hb * n floats each
    std::int64_t diagonal_at = 0;    // inverse_diagonal (float) and inverse_diagonal_f64, n each
    std::int64_t work_at = 0;        // condition-estimate scratch, 4 * n doubles
};

struct PlannerResult {
    double rcond = 0.0;
    double one_norm = 0.0;
    std::int32_t f64 = 0;            // the plan retains Float64
    std::int32_t pad = 0;
};

// Device arrays of a batch (all device pointers).
struct PlannerBatch {
    const PlannerJob *jobs = nullptr;
    int count = 0;
    int max_n = 0;
    const std::uint32_t *offsets = nullptr;
    const std::int32_t *indices = nullptr;
    const double *weights = nullptr;
    double *bands = nullptr;          // G = A^T A, band d at d * n + i
    double *factor = nullptr;         // LDL^T in place of a copy of G
    float *lower = nullptr;
    float *upper = nullptr;
    float *inv_diag = nullptr;
    double *inv_diag64 = nullptr;
    double *work = nullptr;
    PlannerResult *results = nullptr;
};

// Enqueues the planning kernels of `batch` on `stream`; returns a
// cudaError_t value.
int launch_device_planner(const PlannerBatch &batch, void *stream);

} // namespace dsmvc_gb
