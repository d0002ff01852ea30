/*
 * CPU oracle for the descale hot path: test infrastructure only.
 *
 * A plain-C restatement of the reference's inverse-only axis planner and of
 * its CPU scalar execution routes.  Tests, the smoke check and the CPU
 * baseline leg of the benchmark load it to check the CUDA path; the shipped
 * library never links, calls or loads it.
 *
 * Pinned against the reference's own golden vectors (plan and output
 * FNV-1a hashes of tests/numerical_conformance.hpp:126-176, the QR anchor of
 * tests/numerical_contract_tests.cpp:697-728 and the 60-digit bilinear anchor
 * of tests/engine_tests.cpp:992-1026) and against the reference CPU engine
 * compiled from its own sources (oracle/ref).
 */
#ifndef DSMVC_ORACLE_H
#define DSMVC_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Kernel kinds, border modes and precision modes use the reference's enum
 * values (include/dsmvc/engine.hpp:16-60). */
enum { ORC_BILINEAR = 0, ORC_BICUBIC, ORC_LANCZOS, ORC_SPLINE16, ORC_SPLINE36,
       ORC_SPLINE64, ORC_CUSTOM };
enum { ORC_ZERO = 0, ORC_REPEAT, ORC_REFLECT101, ORC_SYMMETRIC, ORC_MIRROR };
enum { ORC_F64_AUTO = 0, ORC_F64_OFF = 1, ORC_F64_FORCE = 2 };

enum {
    ORC_OK = 0,
    ORC_INVALID = 1,   /* std::invalid_argument */
    ORC_RUNTIME = 2,   /* std::runtime_error (incl. non-finite F64 data) */
    ORC_LENGTH = 3,    /* std::length_error / out_of_range */
    ORC_NOMEM = 4
};

typedef double (*orc_custom_fn)(double x, void *user);

typedef struct orc_request {
    int32_t source_size;
    int32_t destination_size;
    double active_length;
    double shift;
    int32_t kind;
    int32_t taps;
    double b;
    double c;
    double blur;
    int32_t border;
    int32_t f64_mode;
} orc_request;

typedef struct orc_conversion {
    float input_offset;
    float input_scale;
    float output_scale;
    float output_offset;
    uint32_t output_maximum;
} orc_conversion;

typedef struct orc_plan {
    int32_t source_size;
    int32_t destination_size;
    int32_t support;
    int32_t half_bandwidth;
    double active_length;
    double shift;
    double normal_rcond;
    double normal_inf_norm;
    size_t nnz;
    uint32_t *transpose_offsets;   /* n + 1 */
    int32_t *transpose_indices;    /* nnz */
    float *transpose_weights;      /* nnz */
    float *lower_ld;               /* hb * n */
    float *upper_l;                /* hb * n */
    float *inverse_diagonal;       /* n */
    int32_t has_f64;
    double *transpose_weights_f64; /* nnz or NULL */
    double *normal_bands_f64;      /* (hb + 1) * n or NULL */
    double *ldlt_bands_f64;        /* (hb + 1) * n or NULL */
    double *inverse_diagonal_f64;  /* n or NULL */
} orc_plan;

int orc_plan_build(const orc_request *request, orc_custom_fn custom,
                   void *user, orc_plan **out);
void orc_plan_free(orc_plan *plan);

uint64_t orc_f32_plan_hash(const orc_request *request, const orc_plan *plan);
uint64_t orc_complete_plan_hash(const orc_request *request,
                                const orc_plan *plan);
uint64_t orc_output_hash_f32(const float *values, size_t count);
uint64_t orc_output_hash_f64(const double *values, size_t count);
void orc_make_normal_input(float *values, size_t count, uint32_t seed);
int32_t orc_padding_index(int64_t index, int32_t size, int32_t mode);

/* Single-axis solves (src/axis_plan.cpp). */
int orc_inverse_axis_f32(const orc_plan *plan, const float *input,
                         ptrdiff_t input_stride, float *output,
                         ptrdiff_t output_stride);
void orc_inverse_axis_f32_ordered(const orc_plan *plan, const float *input,
                                  ptrdiff_t input_stride, float *output,
                                  ptrdiff_t output_stride);
void orc_inverse_axis_f64(const orc_plan *plan, const double *input,
                          ptrdiff_t input_stride, double *output,
                          ptrdiff_t output_stride);
void orc_inverse_axis_f64_ordered(const orc_plan *plan, const double *input,
                                  ptrdiff_t input_stride, double *output,
                                  ptrdiff_t output_stride);

/* The reference CUDA kernels' Float32 operation order (fmaf chains,
 * src/cuda/dsmvc_cuda.cu:62-148), per axis and composed in 2D; kind 0 float,
 * 1 u8, 2 u16. */
void orc_inverse_axis_f32_gpu(const orc_plan *plan, const float *input,
                              ptrdiff_t input_stride, float *output,
                              ptrdiff_t output_stride);
int orc_inverse_2d_gpu_order(const orc_plan *horizontal,
                             const orc_plan *vertical, int kind,
                             const void *input, ptrdiff_t input_stride,
                             void *output, ptrdiff_t output_stride,
                             const orc_conversion *conversion);

/* CpuExecutor(CpuPath::scalar) routes (src/cpu_executor.cpp). Strides are
 * in samples. */
int orc_inverse_rows(const orc_plan *plan, const float *input,
                     ptrdiff_t input_stride, float *output,
                     ptrdiff_t output_stride, int32_t rows);
int orc_inverse_columns(const orc_plan *plan, const float *input,
                        ptrdiff_t input_stride, float *output,
                        ptrdiff_t output_stride, int32_t columns);
int orc_inverse_2d(const orc_plan *horizontal, const orc_plan *vertical,
                   const float *input, ptrdiff_t input_stride, float *output,
                   ptrdiff_t output_stride);
int orc_inverse_2d_u8(const orc_plan *horizontal, const orc_plan *vertical,
                      const uint8_t *input, ptrdiff_t input_stride,
                      uint8_t *output, ptrdiff_t output_stride,
                      const orc_conversion *conversion);
int orc_inverse_2d_u16(const orc_plan *horizontal, const orc_plan *vertical,
                       const uint16_t *input, ptrdiff_t input_stride,
                       uint16_t *output, ptrdiff_t output_stride,
                       const orc_conversion *conversion);

#ifdef __cplusplus
}
#endif

#endif
