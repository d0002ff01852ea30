// Generic-stride axis kernels: one thread solves one vector (a row or a
// column) through the gather, the forward and the backward substitution.
// They serve every layout and every half-bandwidth, and are the
// reference-order baseline the streaming kernels (stream_impl.cuh,
// tstream_impl.cuh) are checked against.
//
// Float32 arithmetic per element is that of the reference CUDA kernels
// (src/cuda/dsmvc_cuda.cu:62-148, inverse_axis_ring): the A^T gather is one
// fmaf chain in CSR order; forward  y_i = (b_i - sum_{d=hb..1} lower*y_{i-d})
// * inv_diag_i with fmaf; backward  x_i = y_i - sum upper*x_{i+d}, the sum an
// fmaf chain in ascending distance for half-bandwidth 3 and descending
// otherwise.
//
// Float64 arithmetic is that of the CPU scalar route (src/axis_plan.cpp:
// 793-823 and 1193-1257) with explicitly rounded __dmul_rn/__dadd_rn/
// __dsub_rn/__ddiv_rn, so that no multiply-add is contracted and the
// results equal the CPU's bit for bit.
#include "kernels.cuh"

#include <cuda_runtime.h>

#include <cfloat>
#include <cstdint>

namespace dsmvc_gb {
namespace {

using dev::AxisJob;
using dev::Conversion;
using dev::PlanView;

__device__ __forceinline__ int find_job(const AxisJob *jobs, int count, int block) {
    int lo = 0, hi = count - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (jobs[mid].first_block <= block) lo = mid; else hi = mid - 1;
    }
    return lo;
}

template <class T> __device__ __forceinline__ float load_f32(const T *p, const Conversion &c) {
    return (static_cast<float>(*p) - c.in_offset) * c.in_scale;
}
template <> __device__ __forceinline__ float load_f32<float>(const float *p, const Conversion &) {
    return *p;
}

template <class T> __device__ __forceinline__ void store_f32(T *p, float v, const Conversion &c) {
    // clamp(v * scale + offset, 0, max) rounded to nearest even, the CPU
    // order (src/cpu_executor.cpp:1919-1939) without contraction.
    float s = __fadd_rn(__fmul_rn(v, c.out_scale), c.out_offset);
    s = fminf(fmaxf(s, 0.0f), static_cast<float>(c.out_max));
    *p = static_cast<T>(__float2uint_rn(s));
}
template <> __device__ __forceinline__ void store_f32<float>(float *p, float v, const Conversion &) {
    *p = v;
}

template <int HB>
__device__ __forceinline__ void shift_ring(float (&r)[HB > 0 ? HB : 1], float v) {
#pragma unroll
    for (int d = HB - 1; d > 0; --d) r[d] = r[d - 1];
    r[0] = v;
}

// HB > 0: fixed half-bandwidth with a register ring; HB == 0: any width,
// previous values re-read from `fwd`.
template <int HB, class In, class Out>
__global__ void __launch_bounds__(128)
axis_f32_kernel(const AxisJob *__restrict__ jobs, int job_count) {
    const int j = find_job(jobs, job_count, static_cast<int>(blockIdx.x));
    const AxisJob &job = jobs[j];
    const int v = (static_cast<int>(blockIdx.x) - job.first_block) * blockDim.x + threadIdx.x;
    if (v >= job.vectors) return;
    const PlanView &p = job.plan;
    const int n = p.destination_size;
    const int hb = HB > 0 ? HB : p.half_bandwidth;
    const In *in = static_cast<const In *>(job.in) + v * job.in_vec;
    float *fwd = static_cast<float *>(job.fwd) + v * job.fwd_vec;
    Out *out = static_cast<Out *>(job.out) + v * job.out_vec;
    const std::int64_t ie = job.in_elem, fe = job.fwd_elem, oe = job.out_elem;
    const Conversion conv = job.conv;

    float ring[HB > 0 ? HB : 1];
#pragma unroll
    for (int d = 0; d < (HB > 0 ? HB : 1); ++d) ring[d] = 0.0f;

    for (int i = 0; i < n; ++i) {
        float sum = 0.0f;
        const std::uint32_t b = __ldg(p.offsets + i), e = __ldg(p.offsets + i + 1);
        for (std::uint32_t k = b; k < e; ++k) {
            sum = fmaf(__ldg(p.weights + k), load_f32(in + __ldg(p.indices + k) * ie, conv), sum);
        }
        if constexpr (HB > 0) {
#pragma unroll
            for (int d = HB; d >= 1; --d) {
                if (d <= i) sum = fmaf(-__ldg(p.lower + (d - 1) * n + i), ring[d - 1], sum);
            }
        } else {
            for (int d = min(hb, i); d >= 1; --d) {
                sum = fmaf(-__ldg(p.lower + (d - 1) * n + i), fwd[(i - d) * fe], sum);
            }
        }
        const float y = sum * __ldg(p.inv_diag + i);
        fwd[i * fe] = y;
        if constexpr (HB > 0) shift_ring<HB>(ring, y);
    }

    // Backward substitution from the last element.
    float last = fwd[(n - 1) * fe];
    store_f32(out + (n - 1) * oe, last, conv);
    if constexpr (HB > 0) {
#pragma unroll
        for (int d = 0; d < HB; ++d) ring[d] = 0.0f;
        ring[0] = last;
    }
    for (int i = n - 2; i >= 0; --i) {
        const int avail = min(hb, n - i - 1);
        float sum = 0.0f;
        if constexpr (HB > 0) {
            if constexpr (HB == 3) {
#pragma unroll
                for (int d = 1; d <= HB; ++d)
                    if (d <= avail) sum = fmaf(__ldg(p.upper + (d - 1) * n + i), ring[d - 1], sum);
            } else {
#pragma unroll
                for (int d = HB; d >= 1; --d)
                    if (d <= avail) sum = fmaf(__ldg(p.upper + (d - 1) * n + i), ring[d - 1], sum);
            }
        } else {
            if (hb == 3) {
                for (int d = 1; d <= avail; ++d)
                    sum = fmaf(__ldg(p.upper + (d - 1) * n + i), fwd[(i + d) * fe], sum);
            } else {
                for (int d = avail; d >= 1; --d)
                    sum = fmaf(__ldg(p.upper + (d - 1) * n + i), fwd[(i + d) * fe], sum);
            }
        }
        const float x = fwd[i * fe] - sum;
        if constexpr (HB == 0) fwd[i * fe] = x;   // later rows read it back
        store_f32(out + i * oe, x, conv);
        if constexpr (HB > 0) shift_ring<HB>(ring, x);
    }
}

// ---- Float64 route ------------------------------------------------------

template <class T> __device__ __forceinline__ double load_f64(const T *p, const Conversion &c) {
    return __dmul_rn(__dsub_rn(static_cast<double>(*p), static_cast<double>(c.in_offset)),
                     static_cast<double>(c.in_scale));
}
template <> __device__ __forceinline__ double load_f64<float>(const float *p, const Conversion &) {
    return static_cast<double>(*p);
}
template <> __device__ __forceinline__ double load_f64<double>(const double *p, const Conversion &) {
    return *p;
}

template <class T>
__device__ __forceinline__ void store_f64(T *p, double v, const Conversion &c, std::uint32_t &flags) {
    // src/cpu_executor.cpp:1617-1645
    const double s = __dadd_rn(__dmul_rn(v, static_cast<double>(c.out_scale)),
                               static_cast<double>(c.out_offset));
    if (!isfinite(v) || !isfinite(s)) {
        flags |= dev::kStatusNonFiniteOutput;
        *p = T{};
        return;
    }
    const double cl = fmin(fmax(s, 0.0), static_cast<double>(c.out_max));
    *p = static_cast<T>(__double2uint_rn(cl));
}
template <>
__device__ __forceinline__ void store_f64<float>(float *p, double v, const Conversion &, std::uint32_t &flags) {
    const float f = __double2float_rn(v);
    if (!isfinite(v) || !isfinite(f)) flags |= dev::kStatusNonFiniteOutput;
    *p = f;
}
template <>
__device__ __forceinline__ void store_f64<double>(double *p, double v, const Conversion &, std::uint32_t &) {
    *p = v;
}

template <class T> __device__ __forceinline__ bool finite_input(T) { return true; }
template <> __device__ __forceinline__ bool finite_input<float>(float v) { return isfinite(v); }

template <int HB>
__device__ __forceinline__ void shift_ring64(double (&r)[HB > 0 ? HB : 1], double v) {
#pragma unroll
    for (int d = HB - 1; d > 0; --d) r[d] = r[d - 1];
    r[0] = v;
}

// Plans that retain Float64 run solve_banded_ldlt (unit-L forward on the
// undivided values, division by D + DBL_EPSILON, backward subtracting term by
// term).  Float32 plans in the Float64 route use their promoted Float32
// factors the way detail::inverse_axis_f64 does (forward with lower*D folded
// in and a multiply by inv_diag; backward summing first, then subtracting).
// HB > 0 keeps the last HB values in registers; HB == 0 re-reads them from
// `fwd` (which then holds z during the forward pass, as the CPU does).
template <int HB, class In, class Out>
__global__ void __launch_bounds__(128)
axis_f64_kernel(const AxisJob *__restrict__ jobs, int job_count, std::uint32_t *status) {
    constexpr int R = HB > 0 ? HB : 1;
    const int j = find_job(jobs, job_count, static_cast<int>(blockIdx.x));
    const AxisJob &job = jobs[j];
    const int v = (static_cast<int>(blockIdx.x) - job.first_block) * blockDim.x + threadIdx.x;
    if (v >= job.vectors) return;
    const PlanView &p = job.plan;
    const int n = p.destination_size;
    const int hb = HB > 0 ? HB : p.half_bandwidth;
    const bool retained = p.retains_f64 != 0;
    const In *in = static_cast<const In *>(job.in) + v * job.in_vec;
    double *fwd = static_cast<double *>(job.fwd) + v * job.fwd_vec;
    Out *out = static_cast<Out *>(job.out) + v * job.out_vec;
    const std::int64_t ie = job.in_elem, fe = job.fwd_elem, oe = job.out_elem;
    const Conversion conv = job.conv;
    std::uint32_t flags = 0;

    double ring[R];
#pragma unroll
    for (int d = 0; d < R; ++d) ring[d] = 0.0;
    for (int i = 0; i < n; ++i) {
        double sum = 0.0;
        const std::uint32_t b = __ldg(p.offsets + i), e = __ldg(p.offsets + i + 1);
        for (std::uint32_t k = b; k < e; ++k) {
            const In raw = in[__ldg(p.indices + k) * ie];
            if (!finite_input(raw)) flags |= dev::kStatusNonFiniteInput;
            const double w = retained ? __ldg(p.weights64 + k)
                                      : static_cast<double>(__ldg(p.weights + k));
            sum = __dadd_rn(sum, __dmul_rn(w, load_f64(&raw, conv)));
        }
        if constexpr (HB > 0) {
#pragma unroll
            for (int d = HB; d >= 1; --d) {
                if (d <= i) {
                    const double f = retained ? __ldg(p.bands64 + d * n + i - d)
                        : static_cast<double>(__ldg(p.lower + (d - 1) * n + i));
                    sum = __dsub_rn(sum, __dmul_rn(f, ring[d - 1]));
                }
            }
            const double y = retained
                ? __ddiv_rn(sum, __dadd_rn(__ldg(p.bands64 + i), DBL_EPSILON))
                : __dmul_rn(sum, static_cast<double>(__ldg(p.inv_diag + i)));
            fwd[i * fe] = y;
            shift_ring64<HB>(ring, retained ? sum : y);
        } else {
            for (int d = min(hb, i); d >= 1; --d) {
                const double f = retained ? __ldg(p.bands64 + d * n + i - d)
                    : static_cast<double>(__ldg(p.lower + (d - 1) * n + i));
                sum = __dsub_rn(sum, __dmul_rn(f, fwd[(i - d) * fe]));
            }
            fwd[i * fe] = retained ? sum : __dmul_rn(sum, static_cast<double>(__ldg(p.inv_diag + i)));
        }
    }
    if constexpr (HB == 0) {
        if (retained) {
            for (int i = 0; i < n; ++i)
                fwd[i * fe] = __ddiv_rn(fwd[i * fe], __dadd_rn(__ldg(p.bands64 + i), DBL_EPSILON));
        }
    }

    const double last = fwd[(n - 1) * fe];
    store_f64(out + (n - 1) * oe, last, conv, flags);
#pragma unroll
    for (int d = 0; d < R; ++d) ring[d] = 0.0;
    ring[0] = last;
    for (int i = n - 2; i >= 0; --i) {
        const int avail = min(hb, n - i - 1);
        double x;
        if constexpr (HB > 0) {
            if (retained) {
                x = fwd[i * fe];
#pragma unroll
                for (int d = HB; d >= 1; --d)
                    if (d <= avail) x = __dsub_rn(x, __dmul_rn(__ldg(p.bands64 + d * n + i), ring[d - 1]));
            } else {
                double sum = 0.0;
#pragma unroll
                for (int d = HB; d >= 1; --d)
                    if (d <= avail)
                        sum = __dadd_rn(sum, __dmul_rn(static_cast<double>(__ldg(p.upper + (d - 1) * n + i)), ring[d - 1]));
                x = __dsub_rn(fwd[i * fe], sum);
            }
            shift_ring64<HB>(ring, x);
        } else {
            if (retained) {
                x = fwd[i * fe];
                for (int d = avail; d >= 1; --d)
                    x = __dsub_rn(x, __dmul_rn(__ldg(p.bands64 + d * n + i), fwd[(i + d) * fe]));
            } else {
                double sum = 0.0;
                for (int d = avail; d >= 1; --d)
                    sum = __dadd_rn(sum, __dmul_rn(static_cast<double>(__ldg(p.upper + (d - 1) * n + i)),
                                                   fwd[(i + d) * fe]));
                x = __dsub_rn(fwd[i * fe], sum);
            }
            fwd[i * fe] = x;
        }
        store_f64(out + i * oe, x, conv, flags);
    }
    if (flags) atomicOr(status, flags);
}

template <int HB, class In, class Out>
int launch_f32_typed(const AxisJob *jobs, int count, int blocks, int threads, cudaStream_t s) {
    axis_f32_kernel<HB, In, Out><<<blocks, threads, 0, s>>>(jobs, count);
    return static_cast<int>(cudaGetLastError());
}

template <int HB>
int launch_f32_hb(const AxisJob *jobs, int count, int blocks, int threads,
                  dev::Sample in, dev::Sample out, cudaStream_t s) {
    using dev::Sample;
    if (in == Sample::f32 && out == Sample::f32) return launch_f32_typed<HB, float, float>(jobs, count, blocks, threads, s);
    if (in == Sample::u8 && out == Sample::f32) return launch_f32_typed<HB, std::uint8_t, float>(jobs, count, blocks, threads, s);
    if (in == Sample::u16 && out == Sample::f32) return launch_f32_typed<HB, std::uint16_t, float>(jobs, count, blocks, threads, s);
    if (in == Sample::f32 && out == Sample::u8) return launch_f32_typed<HB, float, std::uint8_t>(jobs, count, blocks, threads, s);
    if (in == Sample::f32 && out == Sample::u16) return launch_f32_typed<HB, float, std::uint16_t>(jobs, count, blocks, threads, s);
    return static_cast<int>(cudaErrorInvalidValue);
}

template <int HB, class In, class Out>
int launch_f64_typed(const AxisJob *jobs, int count, int blocks, int threads,
                     std::uint32_t *status, cudaStream_t s) {
    axis_f64_kernel<HB, In, Out><<<blocks, threads, 0, s>>>(jobs, count, status);
    return static_cast<int>(cudaGetLastError());
}

template <int HB>
int launch_f64_hb(const AxisJob *jobs, int count, int blocks, int threads,
                  dev::Sample in, dev::Sample out, std::uint32_t *status, cudaStream_t s) {
    using dev::Sample;
    if (in == Sample::f32 && out == Sample::f64) return launch_f64_typed<HB, float, double>(jobs, count, blocks, threads, status, s);
    if (in == Sample::u8 && out == Sample::f64) return launch_f64_typed<HB, std::uint8_t, double>(jobs, count, blocks, threads, status, s);
    if (in == Sample::u16 && out == Sample::f64) return launch_f64_typed<HB, std::uint16_t, double>(jobs, count, blocks, threads, status, s);
    if (in == Sample::f64 && out == Sample::f32) return launch_f64_typed<HB, double, float>(jobs, count, blocks, threads, status, s);
    if (in == Sample::f64 && out == Sample::u8) return launch_f64_typed<HB, double, std::uint8_t>(jobs, count, blocks, threads, status, s);
    if (in == Sample::f64 && out == Sample::u16) return launch_f64_typed<HB, double, std::uint16_t>(jobs, count, blocks, threads, status, s);
    if (in == Sample::f32 && out == Sample::f32) return launch_f64_typed<HB, float, float>(jobs, count, blocks, threads, status, s);
    return static_cast<int>(cudaErrorInvalidValue);
}

} // namespace

int launch_axis_f32(const dev::AxisJob *jobs, int count, int blocks, int threads,
                    int hb, dev::Sample in, dev::Sample out, void *stream) {
    auto s = static_cast<cudaStream_t>(stream);
    switch (hb) {
    case 1: return launch_f32_hb<1>(jobs, count, blocks, threads, in, out, s);
    case 3: return launch_f32_hb<3>(jobs, count, blocks, threads, in, out, s);
    case 5: return launch_f32_hb<5>(jobs, count, blocks, threads, in, out, s);
    case 7: return launch_f32_hb<7>(jobs, count, blocks, threads, in, out, s);
    case 9: return launch_f32_hb<9>(jobs, count, blocks, threads, in, out, s);
    case 11: return launch_f32_hb<11>(jobs, count, blocks, threads, in, out, s);
    default: return launch_f32_hb<0>(jobs, count, blocks, threads, in, out, s);
    }
}

int launch_axis_f64(const dev::AxisJob *jobs, int count, int blocks, int threads,
                    int hb, dev::Sample in, dev::Sample out, std::uint32_t *status, void *stream) {
    auto s = static_cast<cudaStream_t>(stream);
    switch (hb) {
    case 1: return launch_f64_hb<1>(jobs, count, blocks, threads, in, out, status, s);
    case 3: return launch_f64_hb<3>(jobs, count, blocks, threads, in, out, status, s);
    case 5: return launch_f64_hb<5>(jobs, count, blocks, threads, in, out, status, s);
    case 7: return launch_f64_hb<7>(jobs, count, blocks, threads, in, out, status, s);
    case 9: return launch_f64_hb<9>(jobs, count, blocks, threads, in, out, status, s);
    case 11: return launch_f64_hb<11>(jobs, count, blocks, threads, in, out, status, s);
    default: return launch_f64_hb<0>(jobs, count, blocks, threads, in, out, status, s);
    }
}

} // namespace dsmvc_gb
