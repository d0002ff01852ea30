// Optional Float64 residual refinement of the Float64 2D route
// (DSMVC_GB_F64_REFINE=1), and the conversion of its Float64 result.
//
// A Float64 plan retains the unfactored normal band G = A^T A next to its
// LDL^T factor (include/dsmvc/engine.hpp:96-101: the unfactored normal
// matrix "supports independent high-precision residual evaluation").  After
// an axis pass has produced x for every vector, one refinement step
//
//     r = A^T b - G x,    solve G d = r with the LDL^T factor,    x += d
//
// with the residual evaluated in doubled precision: every product split
// exactly into its rounded value and error (fma), every sum accumulated with
// its rounding error (Knuth's TwoSum), as in the compensated dot product of
// Ogita, Rump and Oishi (2005).  The correction solve runs in plain Float64.
// The substitutions' rounding error -- about cond(G) * DBL_EPSILON of the
// solution, which reaches float32 resolution on ill-conditioned plans --
// shrinks to about (cond(G) * DBL_EPSILON)^2, so the refined x is the exact
// solution of the plan's Float64 system (its weights and band G) to about
// one Float64 rounding.  One thread per vector (the recurrences are serial);
// vector v's elements are at X + k * X_elem + v * X_vec as in the sequential
// kernels.
//
//  * refine64_kernel<HB, In>: AxisJob { in = the pass's input b (In), out =
//    x (double, updated in place), fwd = a Float64 scratch vector per vector
//    for the correction }.
//  * convert64_kernel<Out>: AxisJob { in = Float64 result rows, out = the
//    output rows (Out, with the job's conversion) }, vector = output row,
//    plan.destination_size elements per row; non-finite results set status.
#include "tsolve64_impl.cuh"

namespace dsmvc_gb {
namespace {

// Doubled-precision accumulator: value = hi + lo.
struct Compensated {
    double hi = 0.0, lo = 0.0;
    // += a * b, both rounding errors kept.
    __device__ __forceinline__ void add_product(double a, double b) {
        const double p = __dmul_rn(a, b);
        const double e = fma(a, b, -p);              // a * b - p exactly
        const double s = __dadd_rn(hi, p);
        const double z = __dsub_rn(s, hi);
        const double t = __dadd_rn(__dsub_rn(hi, __dsub_rn(s, z)), __dsub_rn(p, z));   // hi + p - s exactly
        hi = s;
        lo = __dadd_rn(lo, __dadd_rn(t, e));
    }
    __device__ __forceinline__ double value() const { return __dadd_rn(hi, lo); }
};

__device__ __forceinline__ int find_axis_job(const dev::AxisJob *jobs, int count, int block) {
    int lo = 0, hi = count - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (jobs[mid].first_block <= block) lo = mid; else hi = mid - 1;
    }
    return lo;
}

template <int HB, class In>
__global__ void __launch_bounds__(128)
refine64_kernel(const dev::AxisJob *__restrict__ jobs, int job_count, std::uint32_t *status) {
    const int j = find_axis_job(jobs, job_count, static_cast<int>(blockIdx.x));
    const dev::AxisJob &job = jobs[j];
    const int v = (static_cast<int>(blockIdx.x) - job.first_block) * blockDim.x + threadIdx.x;
    if (v >= job.vectors) return;
    const dev::PlanView &p = job.plan;
    const int n = p.destination_size;
    const int hb = HB > 0 ? HB : p.half_bandwidth;
    const In *b = static_cast<const In *>(job.in) + v * job.in_vec;
    double *x = static_cast<double *>(job.out) + v * job.out_vec;
    double *z = static_cast<double *>(job.fwd) + v * job.fwd_vec;
    const std::int64_t ie = job.in_elem, xe = job.out_elem, ze = job.fwd_elem;
    const double *g = p.normal64;      // G band d at d * n + i (i the upper row)
    const double *f = p.bands64;       // unit L off the diagonal, D on band 0
    std::uint32_t flags = 0;
    for (int i = 0; i < n; ++i) {
        Compensated acc;
        const std::uint32_t e0 = __ldg(p.offsets + i), e1 = __ldg(p.offsets + i + 1);
        for (std::uint32_t k = e0; k < e1; ++k) {
            const In raw = b[__ldg(p.indices + k) * ie];
            if (!xfinite(raw)) flags |= dev::kStatusNonFiniteInput;
            acc.add_product(__ldg(p.weights64 + k), xload(raw, job.conv));
        }
        for (int d = hb; d >= 1; --d)
            if (d <= i) acc.add_product(-__ldg(g + static_cast<std::int64_t>(d) * n + (i - d)), x[(i - d) * xe]);
        acc.add_product(-__ldg(g + i), x[i * xe]);
        for (int d = 1; d <= hb && i + d < n; ++d)
            acc.add_product(-__ldg(g + static_cast<std::int64_t>(d) * n + i), x[(i + d) * xe]);
        double r = acc.value();
        // Forward substitution with the unit L.
        for (int d = hb; d >= 1; --d)
            if (d <= i) r = fma(-__ldg(f + static_cast<std::int64_t>(d) * n + (i - d)), z[(i - d) * ze], r);
        z[i * ze] = r;
    }
    for (int i = n - 1; i >= 0; --i) {
        double c = z[i * ze] / (__ldg(f + i) + DBL_EPSILON);
        for (int d = hb; d >= 1; --d)
            if (i + d < n) c = fma(-__ldg(f + static_cast<std::int64_t>(d) * n + i), z[(i + d) * ze], c);
        z[i * ze] = c;
        x[i * xe] += c;
    }
    if (flags) atomicOr(status, flags);
}

template <class Out>
__global__ void __launch_bounds__(128)
convert64_kernel(const dev::AxisJob *__restrict__ jobs, int job_count, std::uint32_t *status) {
    const int lo = find_axis_job(jobs, job_count, static_cast<int>(blockIdx.x));
    const dev::AxisJob &job = jobs[lo];
    const int row = (static_cast<int>(blockIdx.x) - job.first_block) * blockDim.x + threadIdx.x;
    if (row >= job.vectors) return;
    const double *src = static_cast<const double *>(job.in) + row * job.in_vec;
    Out *dst = static_cast<Out *>(job.out) + row * job.out_vec;
    std::uint32_t flags = 0;
    for (int k = 0; k < job.plan.destination_size; ++k)
        dst[k * job.out_elem] = xstore<Out>(src[k * job.in_elem], job.conv, flags);
    if (flags) atomicOr(status, flags);
}

template <int HB>
int refine_in(const dev::AxisJob *jobs, int count, int blocks, int threads, dev::Sample in, std::uint32_t *status,
              cudaStream_t s) {
    using dev::Sample;
    switch (in) {
    case Sample::f32: refine64_kernel<HB, float><<<blocks, threads, 0, s>>>(jobs, count, status); break;
    case Sample::u16: refine64_kernel<HB, std::uint16_t><<<blocks, threads, 0, s>>>(jobs, count, status); break;
    case Sample::u8: refine64_kernel<HB, std::uint8_t><<<blocks, threads, 0, s>>>(jobs, count, status); break;
    case Sample::f64: refine64_kernel<HB, double><<<blocks, threads, 0, s>>>(jobs, count, status); break;
    default: return static_cast<int>(cudaErrorInvalidValue);
    }
    return static_cast<int>(cudaGetLastError());
}

} // namespace

int launch_refine64(const dev::AxisJob *jobs, int count, int blocks, int threads, int half_bandwidth, dev::Sample in,
                    std::uint32_t *status, void *stream) {
    if (threads < 32 || threads > 128 || threads % 32) return static_cast<int>(cudaErrorInvalidValue);
    auto s = static_cast<cudaStream_t>(stream);
    switch (half_bandwidth) {
    case 1: return refine_in<1>(jobs, count, blocks, threads, in, status, s);
    case 3: return refine_in<3>(jobs, count, blocks, threads, in, status, s);
    case 5: return refine_in<5>(jobs, count, blocks, threads, in, status, s);
    case 7: return refine_in<7>(jobs, count, blocks, threads, in, status, s);
    case 9: return refine_in<9>(jobs, count, blocks, threads, in, status, s);
    case 11: return refine_in<11>(jobs, count, blocks, threads, in, status, s);
    default: return refine_in<0>(jobs, count, blocks, threads, in, status, s);
    }
}

int launch_convert64(const dev::AxisJob *jobs, int count, int blocks, int threads, dev::Sample out,
                     std::uint32_t *status, void *stream) {
    if (threads < 32 || threads > 128 || threads % 32) return static_cast<int>(cudaErrorInvalidValue);
    auto s = static_cast<cudaStream_t>(stream);
    using dev::Sample;
    switch (out) {
    case Sample::f32: convert64_kernel<float><<<blocks, threads, 0, s>>>(jobs, count, status); break;
    case Sample::u16: convert64_kernel<std::uint16_t><<<blocks, threads, 0, s>>>(jobs, count, status); break;
    case Sample::u8: convert64_kernel<std::uint8_t><<<blocks, threads, 0, s>>>(jobs, count, status); break;
    default: return static_cast<int>(cudaErrorInvalidValue);
    }
    return static_cast<int>(cudaGetLastError());
}

} // namespace dsmvc_gb
