// Device planner kernels (see gpu_planner.cuh).  Every floating-point
// operation is an explicitly rounded double operation (__dadd_rn, __dsub_rn,
// __dmul_rn, __ddiv_rn; no contraction) in the host planner's order, so the
// band, the factor, the condition estimate and the Float32 arrays equal the
// host planner's bit for bit.  Comparisons and min/max follow std::min /
// std::max / std::clamp (the first argument wins ties; no NaN special
// cases).
//
//  * planner_bands_kernel: one thread per (plan, destination i): the hb + 1
//    entries G(i, i + d) = sum over the common source samples of the A^T
//    rows i and i + d, in ascending source order (src/axis_plan.cpp:628-668).
//  * planner_factor_kernel: one thread per plan: the in-place banded LDL^T
//    with pivot D + DBL_EPSILON (src/axis_plan.cpp:766-791), then the
//    condition estimate -- diagonal dominance, the |L^-1| bound, Hager's
//    1-norm estimate with at most eight banded solves
//    (src/axis_plan.cpp:675-908) -- and the Float64 routing (rcond < 1e-4
//    or forced, :909-940).  Serial recurrences: one thread per plan.
//  * planner_arrays_kernel: one thread per (plan, i): inverse_diagonal,
//    upper_l and lower_ld as float, inverse_diagonal_f64
//    (src/axis_plan.cpp:942-967).
#include "gpu_planner.cuh"

#include <cuda_runtime.h>

#include <cfloat>
#include <cstdint>

namespace dsmvc_gb {
namespace {

constexpr double kPlanEps = DBL_EPSILON;
constexpr double kPlanF64Threshold = 1.0e-4;

__device__ __forceinline__ double dmax(double a, double b) { return a < b ? b : a; }
__device__ __forceinline__ double dmin(double a, double b) { return b < a ? b : a; }

__global__ void planner_bands_kernel(PlannerBatch b) {
    const int p = static_cast<int>(blockIdx.y);
    if (p >= b.count) return;
    const PlannerJob job = b.jobs[p];
    const int i = static_cast<int>(blockIdx.x * blockDim.x + threadIdx.x);
    if (i >= job.n) return;
    const std::uint32_t *off = b.offsets + job.offsets_at;
    const std::int32_t *idx = b.indices + job.entries_at;
    const double *w = b.weights + job.entries_at;
    double *g = b.bands + job.bands_at;
    double *f = b.factor + job.bands_at;
    const int n = job.n, hb = job.hb;
    const int maxd = min(hb, n - i - 1);
    for (int d = 0; d <= hb; ++d) {
        double sum = 0.0;
        if (d <= maxd) {
            std::uint32_t l = off[i], le = off[i + 1];
            std::uint32_t r = off[i + d], re = off[i + d + 1];
            while (l < le && r < re) {
                const int li = idx[l], ri = idx[r];
                if (li < ri) {
                    ++l;
                } else if (ri < li) {
                    ++r;
                } else {
                    sum = __dadd_rn(sum, __dmul_rn(w[l], w[r]));
                    ++l;
                    ++r;
                }
            }
        }
        g[static_cast<std::int64_t>(d) * n + i] = sum;
        f[static_cast<std::int64_t>(d) * n + i] = sum;
    }
}

// Banded LDL^T solve in place (src/axis_plan.cpp:793-823).
__device__ void planner_solve(const double *f, int n, int hb, double *v) {
    for (int i = 0; i < n; ++i) {
        double value = v[i];
        for (int d = min(hb, i); d >= 1; --d)
            value = __dsub_rn(value, __dmul_rn(f[static_cast<std::int64_t>(d) * n + (i - d)], v[i - d]));
        v[i] = value;
    }
    for (int i = 0; i < n; ++i) v[i] = __ddiv_rn(v[i], __dadd_rn(f[i], kPlanEps));
    for (int i = n - 2; i >= 0; --i) {
        double value = v[i];
        for (int d = min(hb, n - i - 1); d >= 1; --d)
            value = __dsub_rn(value, __dmul_rn(f[static_cast<std::int64_t>(d) * n + i], v[i + d]));
        v[i] = value;
    }
}

__global__ void planner_factor_kernel(PlannerBatch b) {
    const int p = static_cast<int>(blockIdx.x * blockDim.x + threadIdx.x);
    if (p >= b.count) return;
    const PlannerJob job = b.jobs[p];
    const int n = job.n, hb = job.hb;
    const double *g = b.bands + job.bands_at;
    double *f = b.factor + job.bands_at;

    // Banded LDL^T in place.
    for (int i = 0; i < n; ++i) {
        const int end = min(hb + 1, n - i);
        const double pivot = __dadd_rn(f[i], kPlanEps);
        for (int d = 1; d < end; ++d) {
            const double m = __ddiv_rn(f[static_cast<std::int64_t>(d) * n + i], pivot);
            for (int o = 0; o < end - d; ++o) {
                double &t = f[static_cast<std::int64_t>(o) * n + (i + d)];
                t = __dsub_rn(t, __dmul_rn(m, f[static_cast<std::int64_t>(d + o) * n + i]));
            }
        }
        const double inv = __ddiv_rn(1.0, pivot);
        for (int d = 1; d < end; ++d) {
            double &t = f[static_cast<std::int64_t>(d) * n + i];
            t = __dmul_rn(t, inv);
        }
    }

    // Stage 1: diagonal dominance of G.
    double *work = b.work + job.work_at;
    double *x = work + n, *y = work + 2 * static_cast<std::int64_t>(n), *z = work + 3 * static_cast<std::int64_t>(n);
    for (int c = 0; c < n; ++c) work[c] = 0.0;
    for (int col = 0; col < n; ++col) {
        work[col] = __dadd_rn(work[col], fabs(g[col]));
        for (int d = 1, e = min(hb, n - col - 1); d <= e; ++d) {
            const double v = fabs(g[static_cast<std::int64_t>(d) * n + col]);
            work[col] = __dadd_rn(work[col], v);
            work[col + d] = __dadd_rn(work[col + d], v);
        }
    }
    PlannerResult out;
    double one_norm = work[0];
    for (int c = 1; c < n; ++c)
        if (one_norm < work[c]) one_norm = work[c];
    out.one_norm = one_norm;
    double margin = __longlong_as_double(0x7ff0000000000000LL);   // +infinity
    for (int row = 0; row < n; ++row)
        margin = dmin(margin, __dsub_rn(__dmul_rn(2.0, fabs(g[row])), work[row]));
    out.rcond = margin > 0.0 && one_norm > 0.0 ? __ddiv_rn(margin, one_norm) : 0.0;

    if (!(out.rcond >= kPlanF64Threshold)) {
        // Stage 2: the |L^-1| bound.
        for (int c = 0; c < n; ++c) work[c] = 1.0;
        double inf_norm = 1.0, diag_norm = 0.0;
        for (int row = 0; row < n; ++row) {
            double sum = 1.0;
            for (int d = 1, e = min(hb, row); d <= e; ++d)
                sum = __dadd_rn(sum, __dmul_rn(fabs(f[static_cast<std::int64_t>(d) * n + (row - d)]), work[row - d]));
            work[row] = sum;
            inf_norm = dmax(inf_norm, sum);
            diag_norm = dmax(diag_norm, __ddiv_rn(1.0, fabs(__dadd_rn(f[row], kPlanEps))));
        }
        for (int c = 0; c < n; ++c) work[c] = 1.0;
        double one = 1.0;
        for (int col = n - 1; col >= 0; --col) {
            double sum = 1.0;
            for (int d = 1, e = min(hb, n - col - 1); d <= e; ++d)
                sum = __dadd_rn(sum, __dmul_rn(fabs(f[static_cast<std::int64_t>(d) * n + col]), work[col + d]));
            work[col] = sum;
            one = dmax(one, sum);
        }
        const double bound = __dmul_rn(__dmul_rn(one, diag_norm), inf_norm);
        if (!(one_norm > 0.0) || !(bound > 0.0) || !isfinite(one_norm) || !isfinite(bound)) {
            out.rcond = 0.0;
        } else {
            const double r = __ddiv_rn(1.0, __dmul_rn(one_norm, bound));
            out.rcond = r < 0.0 ? 0.0 : (1.0 < r ? 1.0 : r);
        }

        if (!(out.rcond >= kPlanF64Threshold)) {
            // Stage 3: Hager's 1-norm estimate of G^-1.
            const double start = __ddiv_rn(1.0, static_cast<double>(n));
            for (int c = 0; c < n; ++c) x[c] = start;
            double estimate = 0.0;
            int previous = n;
            for (int it = 0; it < 8; ++it) {
                for (int c = 0; c < n; ++c) y[c] = x[c];
                planner_solve(f, n, hb, y);
                double next = 0.0;
                for (int c = 0; c < n; ++c) next = __dadd_rn(next, fabs(y[c]));
                estimate = dmax(estimate, next);
                for (int c = 0; c < n; ++c) z[c] = y[c] < 0.0 ? -1.0 : 1.0;
                planner_solve(f, n, hb, z);
                int index = 0;
                for (int c = 1; c < n; ++c)
                    if (fabs(z[index]) < fabs(z[c])) index = c;
                double dot = 0.0;
                for (int c = 0; c < n; ++c) dot = __dadd_rn(dot, __dmul_rn(z[c], x[c]));
                if (index == previous || fabs(z[index]) <= dot) break;
                for (int c = 0; c < n; ++c) x[c] = 0.0;
                x[index] = 1.0;
                previous = index;
            }
            if (!(one_norm > 0.0) || !(estimate > 0.0) || !isfinite(one_norm) || !isfinite(estimate)) {
                out.rcond = 0.0;
            } else {
                const double r = __ddiv_rn(1.0, __dmul_rn(one_norm, estimate));
                out.rcond = r < 0.0 ? 0.0 : (1.0 < r ? 1.0 : r);
            }
        }
    }
    out.f64 = job.mode == 2 || (job.mode == 0 && out.rcond < kPlanF64Threshold) ? 1 : 0;
    b.results[p] = out;
}

__global__ void planner_arrays_kernel(PlannerBatch b) {
    const int p = static_cast<int>(blockIdx.y);
    if (p >= b.count) return;
    const PlannerJob job = b.jobs[p];
    const int i = static_cast<int>(blockIdx.x * blockDim.x + threadIdx.x);
    if (i >= job.n) return;
    const int n = job.n, hb = job.hb;
    const double *f = b.factor + job.bands_at;
    float *lower = b.lower + job.factors_at;
    float *upper = b.upper + job.factors_at;
    const double diagonal = f[i];
    const double inv = __ddiv_rn(1.0, __dadd_rn(diagonal, kPlanEps));
    b.inv_diag[job.diagonal_at + i] = __double2float_rn(inv);
    b.inv_diag64[job.diagonal_at + i] = inv;
    for (int d = 1; d <= hb; ++d) {
        const std::int64_t at = static_cast<std::int64_t>(d - 1) * n + i;
        // upper_l[(d-1) n + i] = L(i + d, i); lower_ld[(d-1) n + i] =
        // L(i, i - d) * D(i - d): zero where the band leaves the matrix.
        upper[at] = d <= n - i - 1 ? __double2float_rn(f[static_cast<std::int64_t>(d) * n + i]) : 0.0f;
        lower[at] = i >= d ? __double2float_rn(__dmul_rn(f[static_cast<std::int64_t>(d) * n + (i - d)], f[i - d]))
                           : 0.0f;
    }
}

} // namespace

int launch_device_planner(const PlannerBatch &batch, void *stream) {
    if (batch.count <= 0) return static_cast<int>(cudaSuccess);
    if (batch.count > 65535 || batch.max_n <= 0) return static_cast<int>(cudaErrorInvalidValue);
    auto s = static_cast<cudaStream_t>(stream);
    constexpr int kThreads = 128;
    const dim3 grid((batch.max_n + kThreads - 1) / kThreads, batch.count);
    planner_bands_kernel<<<grid, kThreads, 0, s>>>(batch);
    if (const cudaError_t e = cudaGetLastError(); e != cudaSuccess) return static_cast<int>(e);
    planner_factor_kernel<<<(batch.count + 63) / 64, 64, 0, s>>>(batch);
    if (const cudaError_t e = cudaGetLastError(); e != cudaSuccess) return static_cast<int>(e);
    planner_arrays_kernel<<<grid, kThreads, 0, s>>>(batch);
    return static_cast<int>(cudaGetLastError());
}

} // namespace dsmvc_gb
