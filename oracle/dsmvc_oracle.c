/*
 * CPU oracle for the descale hot path: test infrastructure only (see the
 * header).  Compiled with -ffp-contract=off -fno-fast-math so that every
 * `a * b + c` rounds twice, as the reference's numerical-contract build does
 * (cmake/numerical_contract.cmake:35-36).  Each function names the reference
 * function it restates; the arithmetic order is kept step for step because
 * the plan and output hashes are bit-exact.
 */
#include "dsmvc_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define ORC_PI 3.141592653589793238462643383279502884

static int32_t imin(int32_t a, int32_t b) { return a < b ? a : b; }

/* ---- Kernel weights: src/axis_plan.cpp:246-344 ------------------------- */

static double round_half_up(double value)
{
    return value < 0.0 ? floor(value + 0.5) : floor(value + 0.49999999999999994);
}

static double sq(double v) { return v * v; }
static double cb(double v) { return v * v * v; }

static double sinc(double value)
{
    if (value == 0.0) return 1.0;
    double scaled = ORC_PI * value;
    return sin(scaled) / scaled;
}

static double filter_weight(const orc_request *r, double distance)
{
    double x = fabs(distance);
    double b = r->b, c = r->c;
    switch (r->kind) {
    case ORC_BILINEAR: {
        const double v = 1.0 - x; /* std::max(1 - x, 0) */
        return v < 0.0 ? 0.0 : v;
    }
    case ORC_BICUBIC:
        if (x < 1.0) {
            return ((12.0 - 9.0 * b - 6.0 * c) * cb(x)
                    + (-18.0 + 12.0 * b + 6.0 * c) * sq(x)
                    + (6.0 - 2.0 * b)) / 6.0;
        }
        if (x < 2.0) {
            return ((-b - 6.0 * c) * cb(x)
                    + (6.0 * b + 30.0 * c) * sq(x)
                    + (-12.0 * b - 48.0 * c) * x
                    + (8.0 * b + 24.0 * c)) / 6.0;
        }
        return 0.0;
    case ORC_LANCZOS:
        return r->taps > 0 && x < (double)r->taps
            ? sinc(x) * sinc(x / (double)r->taps) : 0.0;
    case ORC_SPLINE16:
        if (x < 1.0) return 1.0 - x / 5.0 - 9.0 * sq(x) / 5.0 + cb(x);
        if (x < 2.0) {
            x -= 1.0;
            return -7.0 * x / 15.0 + 4.0 * sq(x) / 5.0 - cb(x) / 3.0;
        }
        return 0.0;
    case ORC_SPLINE36:
        if (x < 1.0) {
            return 1.0 - 3.0 * x / 209.0 - 453.0 * sq(x) / 209.0
                + 13.0 * cb(x) / 11.0;
        }
        if (x < 2.0) {
            x -= 1.0;
            return -156.0 * x / 209.0 + 270.0 * sq(x) / 209.0
                - 6.0 * cb(x) / 11.0;
        }
        if (x < 3.0) {
            x -= 2.0;
            return 26.0 * x / 209.0 - 45.0 * sq(x) / 209.0 + cb(x) / 11.0;
        }
        return 0.0;
    case ORC_SPLINE64:
        if (x < 1.0) {
            return 1.0 - 3.0 * x / 2911.0 - 6387.0 * sq(x) / 2911.0
                + 49.0 * cb(x) / 41.0;
        }
        if (x < 2.0) {
            x -= 1.0;
            return -2328.0 * x / 2911.0 + 4032.0 * sq(x) / 2911.0
                - 24.0 * cb(x) / 41.0;
        }
        if (x < 3.0) {
            x -= 2.0;
            return 582.0 * x / 2911.0 - 1008.0 * sq(x) / 2911.0
                + 6.0 * cb(x) / 41.0;
        }
        if (x < 4.0) {
            x -= 3.0;
            return -97.0 * x / 2911.0 + 168.0 * sq(x) / 2911.0 - cb(x) / 41.0;
        }
        return 0.0;
    default:
        return 0.0;
    }
}

/* src/axis_plan.cpp:370-424 */
static int filter_support(const orc_request *r, int32_t *support)
{
    if (r->source_size <= 0 || r->destination_size <= 0) return ORC_INVALID;
    if (!(r->active_length > 0.0) || !isfinite(r->active_length)
        || !isfinite(r->shift)) return ORC_INVALID;
    if (r->border < ORC_ZERO || r->border > ORC_MIRROR) return ORC_INVALID;
    if (r->f64_mode < 0 || r->f64_mode > 2) return ORC_INVALID;
    if (!(r->blur > 0.0) || !isfinite(r->blur)) return ORC_INVALID;
    int32_t base = 0;
    switch (r->kind) {
    case ORC_BILINEAR: base = 1; break;
    case ORC_BICUBIC: case ORC_SPLINE16: base = 2; break;
    case ORC_SPLINE36: base = 3; break;
    case ORC_SPLINE64: base = 4; break;
    case ORC_LANCZOS: case ORC_CUSTOM: base = r->taps; break;
    default: return ORC_INVALID;
    }
    const int32_t maximum = (INT32_MAX - 1) / 2;
    if (base <= 0 || base > maximum) return ORC_INVALID;
    double scaled = (double)base * r->blur;
    if (!isfinite(scaled) || scaled > (double)maximum) return ORC_LENGTH;
    double effective = ceil(scaled);
    if (!(effective >= 1.0) || effective > (double)maximum) return ORC_LENGTH;
    *support = (int32_t)effective;
    return ORC_OK;
}

/* detail::padding_index, src/axis_plan.cpp:1024-1066 */
int32_t orc_padding_index(int64_t index, int32_t size, int32_t mode)
{
    int64_t extent = size;
    if (index >= 0 && index < extent) return (int32_t)index;
    switch (mode) {
    case ORC_ZERO: return -1;
    case ORC_REPEAT: return index < 0 ? 0 : size - 1;
    case ORC_REFLECT101: {
        if (size == 1) return 0;
        int64_t period = 2 * (extent - 1);
        int64_t mapped = index % period;
        if (mapped < 0) mapped += period;
        return (int32_t)(mapped < extent ? mapped : period - mapped);
    }
    case ORC_SYMMETRIC: {
        int64_t period = 2 * extent;
        int64_t mapped = index % period;
        if (mapped < 0) mapped += period;
        return (int32_t)(mapped < extent ? mapped : period - 1 - mapped);
    }
    case ORC_MIRROR:
        if (index < -extent || index >= 2 * extent) return -1;
        return (int32_t)(index < 0 ? -index - 1 : 2 * extent - index - 1);
    }
    return -1;
}

/* ---- Planner: src/axis_plan.cpp:456-970 -------------------------------- */

typedef struct dcsr {
    uint32_t *offsets;
    int32_t *indices;
    double *weights;
    size_t nnz;
} dcsr;

static void dcsr_free(dcsr *m)
{
    free(m->offsets);
    free(m->indices);
    free(m->weights);
    memset(m, 0, sizeof(*m));
}

static int cmp_i32(const void *a, const void *b)
{
    int32_t x = *(const int32_t *)a, y = *(const int32_t *)b;
    return (x > y) - (x < y);
}

/* build_geometry (:456-518) followed by make_descale_matrix (:535-599): for
 * every source sample, 2*support taps around its position, border-mapped
 * destination indices coalesced into ascending unique columns, weights
 * normalised by the row's tap sum. */
static int make_descale_matrix(const orc_request *r, int32_t support,
                               orc_custom_fn custom, void *user, dcsr *out)
{
    const int32_t taps = 2 * support;
    const int32_t m = r->source_size;
    size_t capacity = (size_t)m * (size_t)taps;
    if (taps != 0 && capacity / (size_t)taps != (size_t)m) return ORC_LENGTH;
    out->offsets = calloc((size_t)m + 1, sizeof(uint32_t));
    out->indices = malloc((capacity ? capacity : 1) * sizeof(int32_t));
    out->weights = malloc((capacity ? capacity : 1) * sizeof(double));
    double *dist = malloc((size_t)taps * sizeof(double));
    double *tw = malloc((size_t)taps * sizeof(double));
    double *coal = malloc((size_t)taps * sizeof(double));
    int32_t *tidx = malloc((size_t)taps * sizeof(int32_t));
    int32_t *uniq = malloc((size_t)taps * sizeof(int32_t));
    int32_t *slot = malloc((size_t)taps * sizeof(int32_t));
    unsigned char *seen = malloc((size_t)taps);
    int status = ORC_OK;
    if (!out->offsets || !out->indices || !out->weights || !dist || !tw
        || !coal || !tidx || !uniq || !slot || !seen) {
        status = ORC_NOMEM;
        goto done;
    }
    const double ratio = (double)r->source_size / r->active_length;
    const int unity_blur = r->blur == 1.0;
    size_t nnz = 0;
    for (int32_t row = 0; row < m; ++row) {
        const double position = ((double)row + 0.5) / ratio + r->shift;
        const double begin = round_half_up(position - (double)support) + 0.5;
        int32_t nuniq = 0;
        for (int32_t t = 0; t < taps; ++t) {
            const double center = begin + (double)t;
            dist[t] = center - position;
            const double fl = floor(center);
            if (!isfinite(fl) || fl < -0x1p63 || fl >= 0x1p63) {
                status = ORC_LENGTH;
                goto done;
            }
            int32_t index = orc_padding_index((int64_t)fl, r->destination_size,
                                              r->border);
            tidx[t] = index;
            if (index >= 0) {
                int found = 0;
                for (int32_t k = 0; k < nuniq; ++k) found |= uniq[k] == index;
                if (!found) uniq[nuniq++] = index;
            }
        }
        qsort(uniq, (size_t)nuniq, sizeof(int32_t), cmp_i32);
        for (int32_t t = 0; t < taps; ++t) {
            slot[t] = -1;
            if (tidx[t] < 0) continue;
            for (int32_t k = 0; k < nuniq; ++k) {
                if (uniq[k] == tidx[t]) { slot[t] = k; break; }
            }
        }
        double total = 0.0;
        for (int32_t t = 0; t < taps; ++t) {
            const double distance = unity_blur ? dist[t] : dist[t] / r->blur;
            const double w = r->kind == ORC_CUSTOM
                ? custom(fabs(distance), user) : filter_weight(r, distance);
            if (!isfinite(w)) { status = ORC_RUNTIME; goto done; }
            tw[t] = w;
            total += w;
        }
        if (!isfinite(total) || total == 0.0) { status = ORC_RUNTIME; goto done; }
        for (int32_t k = 0; k < nuniq; ++k) { coal[k] = 0.0; seen[k] = 0; }
        for (int32_t t = 0; t < taps; ++t) {
            if (slot[t] < 0) continue;
            const double w = tw[t] / total;
            if (w == 0.0) continue;
            coal[slot[t]] += w;
            seen[slot[t]] = 1;
        }
        for (int32_t k = 0; k < nuniq; ++k) {
            if (!seen[k]) continue;
            out->indices[nnz] = uniq[k];
            out->weights[nnz] = coal[k];
            ++nnz;
        }
        if (nnz > UINT32_MAX) { status = ORC_LENGTH; goto done; }
        out->offsets[row + 1] = (uint32_t)nnz;
    }
    out->nnz = nnz;
done:
    free(dist); free(tw); free(coal); free(tidx); free(uniq); free(slot);
    free(seen);
    return status;
}

/* transpose_csr (:601-626): counting sort by destination column; the source
 * rows of every column stay ascending. */
static int transpose_csr(const dcsr *in, int32_t rows, int32_t columns,
                         dcsr *out)
{
    out->nnz = in->nnz;
    out->offsets = calloc((size_t)columns + 1, sizeof(uint32_t));
    out->indices = malloc((in->nnz ? in->nnz : 1) * sizeof(int32_t));
    out->weights = malloc((in->nnz ? in->nnz : 1) * sizeof(double));
    uint32_t *cursor = malloc(((size_t)columns + 1) * sizeof(uint32_t));
    if (!out->offsets || !out->indices || !out->weights || !cursor) {
        free(cursor);
        return ORC_NOMEM;
    }
    for (size_t k = 0; k < in->nnz; ++k) ++out->offsets[in->indices[k] + 1];
    for (int32_t c = 0; c < columns; ++c) out->offsets[c + 1] += out->offsets[c];
    memcpy(cursor, out->offsets, ((size_t)columns + 1) * sizeof(uint32_t));
    for (int32_t row = 0; row < rows; ++row) {
        for (uint32_t k = in->offsets[row]; k < in->offsets[row + 1]; ++k) {
            uint32_t target = cursor[in->indices[k]]++;
            out->indices[target] = row;
            out->weights[target] = in->weights[k];
        }
    }
    free(cursor);
    return ORC_OK;
}

/* form_normal_bands (:628-668): G = A^T A, band d of column i at d*n+i,
 * products accumulated in ascending source order. */
static void form_normal_bands(const dcsr *t, int32_t n, int32_t hb,
                              double *bands)
{
    const size_t w = (size_t)n;
    memset(bands, 0, ((size_t)hb + 1) * w * sizeof(double));
    for (int32_t left_row = 0; left_row < n; ++left_row) {
        const int32_t maxd = imin(hb, n - left_row - 1);
        for (int32_t d = 0; d <= maxd; ++d) {
            const int32_t right_row = left_row + d;
            uint32_t l = t->offsets[left_row], le = t->offsets[left_row + 1];
            uint32_t rr = t->offsets[right_row], re = t->offsets[right_row + 1];
            double sum = 0.0;
            while (l < le && rr < re) {
                int32_t li = t->indices[l], ri = t->indices[rr];
                if (li < ri) {
                    ++l;
                } else if (ri < li) {
                    ++rr;
                } else {
                    sum += t->weights[l] * t->weights[rr];
                    ++l;
                    ++rr;
                }
            }
            bands[(size_t)d * w + (size_t)left_row] = sum;
        }
    }
}

/* symmetric_band_condition_bounds (:675-711) */
static void condition_bounds(const double *bands, int32_t n, int32_t hb,
                             double *work, double *one_norm, double *dd_rcond)
{
    const size_t w = (size_t)n;
    for (int32_t i = 0; i < n; ++i) work[i] = 0.0;
    for (int32_t col = 0; col < n; ++col) {
        work[col] += fabs(bands[col]);
        const int32_t avail = imin(hb, n - col - 1);
        for (int32_t d = 1; d <= avail; ++d) {
            const double v = fabs(bands[(size_t)d * w + (size_t)col]);
            work[col] += v;
            work[col + d] += v;
        }
    }
    double norm = n > 0 ? work[0] : 0.0;
    for (int32_t i = 1; i < n; ++i) if (norm < work[i]) norm = work[i];
    double margin = INFINITY;
    for (int32_t row = 0; row < n; ++row) {
        const double diag = fabs(bands[row]);
        const double v = 2.0 * diag - work[row];
        margin = v < margin ? v : margin;
    }
    *one_norm = norm;
    *dd_rcond = margin > 0.0 && norm > 0.0 ? margin / norm : 0.0;
}

static double clamp01(double v) { return v < 0.0 ? 0.0 : (v > 1.0 ? 1.0 : v); }

/* reciprocal_condition_lower_bound (:713-764) */
static double rcond_lower_bound(double norm, const double *f, int32_t n,
                                int32_t hb, double *work)
{
    const size_t w = (size_t)n;
    const double eps = DBL_EPSILON;
    for (int32_t i = 0; i < n; ++i) work[i] = 1.0;
    double inf_norm = 1.0, diag_norm = 0.0;
    for (int32_t row = 0; row < n; ++row) {
        double sum = 1.0;
        const int32_t avail = imin(hb, row);
        for (int32_t d = 1; d <= avail; ++d) {
            const int32_t col = row - d;
            sum += fabs(f[(size_t)d * w + (size_t)col]) * work[col];
        }
        work[row] = sum;
        inf_norm = inf_norm < sum ? sum : inf_norm;
        const double inv = 1.0 / fabs(f[row] + eps);
        diag_norm = diag_norm < inv ? inv : diag_norm;
    }
    for (int32_t i = 0; i < n; ++i) work[i] = 1.0;
    double one = 1.0;
    for (int32_t col = n - 1; col >= 0; --col) {
        double sum = 1.0;
        const int32_t avail = imin(hb, n - col - 1);
        for (int32_t d = 1; d <= avail; ++d) {
            sum += fabs(f[(size_t)d * w + (size_t)col]) * work[col + d];
        }
        work[col] = sum;
        one = one < sum ? sum : one;
    }
    const double bound = one * diag_norm * inf_norm;
    if (!(norm > 0.0) || !(bound > 0.0) || !isfinite(norm) || !isfinite(bound)) {
        return 0.0;
    }
    return clamp01(1.0 / (norm * bound));
}

/* factor_banded_ldlt (:766-791): in place, pivot D + DBL_EPSILON. */
static void factor_banded_ldlt(double *bands, int32_t n, int32_t hb)
{
    const size_t w = (size_t)n;
    const double eps = DBL_EPSILON;
    for (int32_t i = 0; i < n; ++i) {
        const int32_t end = imin(hb + 1, n - i);
        const double pivot = bands[i] + eps;
        for (int32_t d = 1; d < end; ++d) {
            const double mult = bands[(size_t)d * w + (size_t)i] / pivot;
            for (int32_t o = 0; o < end - d; ++o) {
                bands[(size_t)o * w + (size_t)(i + d)] -=
                    mult * bands[(size_t)(d + o) * w + (size_t)i];
            }
        }
        const double inv = 1.0 / pivot;
        for (int32_t d = 1; d < end; ++d) bands[(size_t)d * w + (size_t)i] *= inv;
    }
}

/* solve_banded_ldlt (:793-823) */
static void solve_banded_ldlt(const double *f, int32_t n, int32_t hb,
                              double *v, ptrdiff_t s)
{
    const size_t w = (size_t)n;
    const double eps = DBL_EPSILON;
    for (int32_t i = 0; i < n; ++i) {
        double value = v[(ptrdiff_t)i * s];
        for (int32_t d = imin(hb, i); d >= 1; --d) {
            value -= f[(size_t)d * w + (size_t)(i - d)] * v[(ptrdiff_t)(i - d) * s];
        }
        v[(ptrdiff_t)i * s] = value;
    }
    for (int32_t i = 0; i < n; ++i) v[(ptrdiff_t)i * s] /= f[i] + eps;
    for (int32_t i = n - 2; i >= 0; --i) {
        double value = v[(ptrdiff_t)i * s];
        for (int32_t d = imin(hb, n - i - 1); d >= 1; --d) {
            value -= f[(size_t)d * w + (size_t)i] * v[(ptrdiff_t)(i + d) * s];
        }
        v[(ptrdiff_t)i * s] = value;
    }
}

/* estimate_inverse_one_norm (:825-861), Hager's method, at most 8 steps. */
static double estimate_inverse_one_norm(const double *f, int32_t n, int32_t hb,
                                        double *x, double *y, double *z)
{
    const size_t size = (size_t)n;
    for (size_t i = 0; i < size; ++i) x[i] = 1.0 / (double)n;
    double estimate = 0.0;
    size_t previous = size;
    for (int it = 0; it < 8; ++it) {
        memcpy(y, x, size * sizeof(double));
        solve_banded_ldlt(f, n, hb, y, 1);
        double next = 0.0;
        for (size_t i = 0; i < size; ++i) next = next + fabs(y[i]);
        estimate = estimate < next ? next : estimate;
        for (size_t i = 0; i < size; ++i) z[i] = y[i] < 0.0 ? -1.0 : 1.0;
        solve_banded_ldlt(f, n, hb, z, 1);
        size_t index = 0;
        for (size_t i = 1; i < size; ++i) if (fabs(z[index]) < fabs(z[i])) index = i;
        double dot = 0.0;
        for (size_t i = 0; i < size; ++i) dot = dot + z[i] * x[i];
        if (index == previous || fabs(z[index]) <= dot) break;
        for (size_t i = 0; i < size; ++i) x[i] = 0.0;
        x[index] = 1.0;
        previous = index;
    }
    return estimate;
}

void orc_plan_free(orc_plan *p)
{
    if (!p) return;
    free(p->transpose_offsets);
    free(p->transpose_indices);
    free(p->transpose_weights);
    free(p->lower_ld);
    free(p->upper_l);
    free(p->inverse_diagonal);
    free(p->transpose_weights_f64);
    free(p->normal_bands_f64);
    free(p->ldlt_bands_f64);
    free(p->inverse_diagonal_f64);
    free(p);
}

/* build_axis_plan_impl (:875-970) */
int orc_plan_build(const orc_request *r, orc_custom_fn custom, void *user,
                   orc_plan **out)
{
    *out = NULL;
    int32_t support = 0;
    int status = filter_support(r, &support);
    if (status) return status;
    if (r->kind == ORC_CUSTOM && !custom) return ORC_INVALID;
    dcsr a = {0}, t = {0};
    status = make_descale_matrix(r, support, custom, user, &a);
    if (status) { dcsr_free(&a); return status; }
    const int32_t n = r->destination_size;
    status = transpose_csr(&a, r->source_size, n, &t);
    dcsr_free(&a);
    if (status) { dcsr_free(&t); return status; }
    const int32_t hb = imin(2 * support - 1, n - 1);
    const size_t w = (size_t)n;
    const size_t band_count = ((size_t)hb + 1) * w;
    double *normal = malloc(band_count * sizeof(double));
    double *factors = malloc(band_count * sizeof(double));
    double *work = malloc(w * 3 * sizeof(double) + sizeof(double));
    orc_plan *p = calloc(1, sizeof(orc_plan));
    if (!normal || !factors || !work || !p) {
        free(normal); free(factors); free(work); free(p); dcsr_free(&t);
        return ORC_NOMEM;
    }
    form_normal_bands(&t, n, hb, normal);
    memcpy(factors, normal, band_count * sizeof(double));
    factor_banded_ldlt(factors, n, hb);

    const double threshold = 1.0e-4;
    double one_norm = 0.0, rcond = 0.0;
    condition_bounds(normal, n, hb, work, &one_norm, &rcond);
    if (rcond < threshold) {
        rcond = rcond_lower_bound(one_norm, factors, n, hb, work);
        if (rcond < threshold) {
            double inv = estimate_inverse_one_norm(factors, n, hb, work,
                                                   work + w, work + 2 * w);
            if (!(one_norm > 0.0) || !(inv > 0.0) || !isfinite(one_norm)
                || !isfinite(inv)) {
                rcond = 0.0;
            } else {
                rcond = clamp01(1.0 / (one_norm * inv));
            }
        }
    }
    const int f64 = r->f64_mode == ORC_F64_FORCE
        || (r->f64_mode == ORC_F64_AUTO && rcond < threshold);

    p->source_size = r->source_size;
    p->destination_size = n;
    p->support = support;
    p->half_bandwidth = hb;
    p->active_length = r->active_length;
    p->shift = r->shift;
    p->normal_rcond = rcond;
    p->nnz = t.nnz;
    p->transpose_offsets = t.offsets;
    p->transpose_indices = t.indices;
    p->transpose_weights = malloc((t.nnz ? t.nnz : 1) * sizeof(float));
    p->lower_ld = calloc((size_t)hb * w + 1, sizeof(float));
    p->upper_l = calloc((size_t)hb * w + 1, sizeof(float));
    p->inverse_diagonal = malloc(w * sizeof(float));
    if (!p->transpose_weights || !p->lower_ld || !p->upper_l
        || !p->inverse_diagonal) {
        free(normal); free(factors); free(work); free(t.weights);
        orc_plan_free(p);
        return ORC_NOMEM;
    }
    for (size_t k = 0; k < t.nnz; ++k) p->transpose_weights[k] = (float)t.weights[k];
    if (f64) {
        p->has_f64 = 1;
        p->normal_inf_norm = one_norm;
        p->transpose_weights_f64 = t.weights;
        t.weights = NULL;
        p->normal_bands_f64 = normal;
        normal = NULL;
        p->ldlt_bands_f64 = malloc(band_count * sizeof(double));
        p->inverse_diagonal_f64 = malloc(w * sizeof(double));
        memcpy(p->ldlt_bands_f64, factors, band_count * sizeof(double));
        for (int32_t i = 0; i < n; ++i) {
            p->inverse_diagonal_f64[i] = 1.0 / (factors[i] + DBL_EPSILON);
        }
    }
    for (int32_t i = 0; i < n; ++i) {
        const double diagonal = factors[i];
        p->inverse_diagonal[i] = (float)(1.0 / (diagonal + DBL_EPSILON));
        const int32_t avail = imin(hb, n - i - 1);
        for (int32_t d = 1; d <= avail; ++d) {
            const double l = factors[(size_t)d * w + (size_t)i];
            p->upper_l[(size_t)(d - 1) * w + (size_t)i] = (float)l;
            p->lower_ld[(size_t)(d - 1) * w + (size_t)(i + d)] =
                (float)(l * diagonal);
        }
    }
    free(normal);
    free(factors);
    free(work);
    free(t.weights);
    /* AxisPlan::check_valid (:1259-1341): only finiteness can fail here. */
    for (size_t k = 0; k < (size_t)hb * w; ++k) {
        if (!isfinite(p->lower_ld[k]) || !isfinite(p->upper_l[k])) {
            orc_plan_free(p);
            return ORC_RUNTIME;
        }
    }
    for (int32_t i = 0; i < n; ++i) {
        if (!isfinite(p->inverse_diagonal[i])) {
            orc_plan_free(p);
            return ORC_RUNTIME;
        }
    }
    *out = p;
    return ORC_OK;
}

/* ---- Stable FNV-1a hashes: tests/numerical_conformance.hpp:22-80 -------- */

typedef struct hasher { uint64_t v; } hasher;

static void h_mix(hasher *h, uint8_t byte)
{
    h->v ^= byte;
    h->v *= 1099511628211ULL;
}
static void h_uint(hasher *h, uint64_t value, size_t bytes)
{
    for (size_t i = 0; i < bytes; ++i) {
        h_mix(h, (uint8_t)(value & 0xffU));
        value >>= 8U;
    }
}
static void h_str(hasher *h, const char *s)
{
    size_t len = strlen(s);
    h_uint(h, (uint64_t)len, 8);
    for (size_t i = 0; i < len; ++i) h_mix(h, (uint8_t)s[i]);
}
static void h_f64(hasher *h, double v)
{
    uint64_t bits;
    memcpy(&bits, &v, 8);
    h_uint(h, bits, 8);
}
static void h_f32(hasher *h, float v)
{
    uint32_t bits;
    memcpy(&bits, &v, 4);
    h_uint(h, bits, 4);
}
static void h_i32(hasher *h, int32_t v) { h_uint(h, (uint32_t)v, 4); }
static void h_u8(hasher *h, uint8_t v) { h_uint(h, v, 1); }

static void h_request_plan_head(hasher *h, const orc_request *r,
                                const orc_plan *p)
{
    h_i32(h, r->source_size);
    h_i32(h, r->destination_size);
    h_f64(h, r->active_length);
    h_f64(h, r->shift);
    h_u8(h, (uint8_t)r->kind);
    h_i32(h, r->taps);
    h_f64(h, r->b);
    h_f64(h, r->c);
    h_u8(h, (uint8_t)r->border);
    h_u8(h, (uint8_t)r->f64_mode);
    h_i32(h, p->source_size);
    h_i32(h, p->destination_size);
    h_i32(h, p->support);
    h_i32(h, p->half_bandwidth);
    h_f64(h, p->active_length);
    h_f64(h, p->shift);
}

static void h_f32_arrays(hasher *h, const orc_plan *p)
{
    const size_t n = (size_t)p->destination_size;
    const size_t f = (size_t)p->half_bandwidth * n;
    h_uint(h, (uint64_t)(n + 1), 8);
    for (size_t i = 0; i <= n; ++i) h_uint(h, p->transpose_offsets[i], 4);
    h_uint(h, (uint64_t)p->nnz, 8);
    for (size_t i = 0; i < p->nnz; ++i) h_i32(h, p->transpose_indices[i]);
    h_uint(h, (uint64_t)p->nnz, 8);
    for (size_t i = 0; i < p->nnz; ++i) h_f32(h, p->transpose_weights[i]);
    h_uint(h, (uint64_t)f, 8);
    for (size_t i = 0; i < f; ++i) h_f32(h, p->lower_ld[i]);
    h_uint(h, (uint64_t)f, 8);
    for (size_t i = 0; i < f; ++i) h_f32(h, p->upper_l[i]);
    h_uint(h, (uint64_t)n, 8);
    for (size_t i = 0; i < n; ++i) h_f32(h, p->inverse_diagonal[i]);
}

static void h_f64_span(hasher *h, const double *v, size_t count)
{
    h_uint(h, (uint64_t)count, 8);
    for (size_t i = 0; i < count; ++i) h_f64(h, v[i]);
}

uint64_t orc_f32_plan_hash(const orc_request *r, const orc_plan *p)
{
    hasher h = {1469598103934665603ULL};
    h_str(&h, "dsmvc-f32-axis-plan-v1");
    h_request_plan_head(&h, r, p);
    h_u8(&h, p->normal_rcond < 1.0e-4 ? 1 : 0);
    h_u8(&h, p->has_f64 ? 1 : 0);
    h_f32_arrays(&h, p);
    return h.v;
}

uint64_t orc_complete_plan_hash(const orc_request *r, const orc_plan *p)
{
    hasher h = {1469598103934665603ULL};
    h_str(&h, "dsmvc-axis-plan-v1");
    h_request_plan_head(&h, r, p);
    h_f64(&h, p->normal_rcond);
    h_f64(&h, p->normal_inf_norm);
    h_f32_arrays(&h, p);
    const size_t n = (size_t)p->destination_size;
    const size_t bands = ((size_t)p->half_bandwidth + 1) * n;
    h_f64_span(&h, p->transpose_weights_f64, p->has_f64 ? p->nnz : 0);
    h_f64_span(&h, p->normal_bands_f64, p->has_f64 ? bands : 0);
    h_f64_span(&h, p->ldlt_bands_f64, p->has_f64 ? bands : 0);
    h_f64_span(&h, p->inverse_diagonal_f64, p->has_f64 ? n : 0);
    return h.v;
}

uint64_t orc_output_hash_f32(const float *v, size_t count)
{
    hasher h = {1469598103934665603ULL};
    h_str(&h, "dsmvc-ordered-output-v1");
    h_uint(&h, (uint64_t)count, 8);
    for (size_t i = 0; i < count; ++i) h_f32(&h, v[i]);
    return h.v;
}

uint64_t orc_output_hash_f64(const double *v, size_t count)
{
    hasher h = {1469598103934665603ULL};
    h_str(&h, "dsmvc-ordered-output-v1");
    h_f64_span(&h, v, count);
    return h.v;
}

/* make_normal_input, tests/numerical_conformance.hpp:178-191 */
void orc_make_normal_input(float *values, size_t count, uint32_t seed)
{
    uint32_t state = seed;
    for (size_t i = 0; i < count; ++i) {
        state ^= state << 13U;
        state ^= state >> 17U;
        state ^= state << 5U;
        uint32_t bits = 0x3f000000U | (state & 0x007fffffU);
        if (state & 0x00800000U) bits |= 0x80000000U;
        memcpy(&values[i], &bits, 4);
    }
}

/* ---- Axis solves ------------------------------------------------------- */

/* inverse_axis_impl (src/axis_plan.cpp:973-1018): gather in CSR order, then
 * forward substitution (descending distance) and the backward pass that sums
 * first (ascending distance for half-bandwidth 3, descending otherwise). */
static void inverse_axis_f32_scalar(const orc_plan *p, const float *in,
                                    ptrdiff_t is, float *out, ptrdiff_t os)
{
    const int32_t n = p->destination_size, hb = p->half_bandwidth;
    const size_t w = (size_t)n;
    for (int32_t i = 0; i < n; ++i) {
        float sum = 0.0f;
        for (uint32_t k = p->transpose_offsets[i]; k < p->transpose_offsets[i + 1]; ++k) {
            sum += p->transpose_weights[k] * in[(ptrdiff_t)p->transpose_indices[k] * is];
        }
        for (int32_t d = imin(hb, i); d >= 1; --d) {
            sum -= p->lower_ld[(size_t)(d - 1) * w + (size_t)i]
                * out[(ptrdiff_t)(i - d) * os];
        }
        out[(ptrdiff_t)i * os] = sum * p->inverse_diagonal[i];
    }
    for (int32_t i = n - 2; i >= 0; --i) {
        float sum = 0.0f;
        const int32_t avail = imin(hb, n - i - 1);
        if (hb == 3) {
            for (int32_t d = 1; d <= avail; ++d) {
                sum += p->upper_l[(size_t)(d - 1) * w + (size_t)i]
                    * out[(ptrdiff_t)(i + d) * os];
            }
        } else {
            for (int32_t d = avail; d >= 1; --d) {
                sum += p->upper_l[(size_t)(d - 1) * w + (size_t)i]
                    * out[(ptrdiff_t)(i + d) * os];
            }
        }
        out[(ptrdiff_t)i * os] -= sum;
    }
}

/* detail::inverse_axis_f64 (:1193-1257) */
void orc_inverse_axis_f64(const orc_plan *p, const double *in, ptrdiff_t is,
                          double *out, ptrdiff_t os)
{
    const int32_t n = p->destination_size, hb = p->half_bandwidth;
    const size_t w = (size_t)n;
    if (p->has_f64) {
        for (int32_t i = 0; i < n; ++i) {
            double sum = 0.0;
            for (uint32_t k = p->transpose_offsets[i]; k < p->transpose_offsets[i + 1]; ++k) {
                sum += p->transpose_weights_f64[k]
                    * in[(ptrdiff_t)p->transpose_indices[k] * is];
            }
            out[(ptrdiff_t)i * os] = sum;
        }
        solve_banded_ldlt(p->ldlt_bands_f64, n, hb, out, os);
        return;
    }
    for (int32_t i = 0; i < n; ++i) {
        double sum = 0.0;
        for (uint32_t k = p->transpose_offsets[i]; k < p->transpose_offsets[i + 1]; ++k) {
            sum += (double)p->transpose_weights[k]
                * in[(ptrdiff_t)p->transpose_indices[k] * is];
        }
        for (int32_t d = imin(hb, i); d >= 1; --d) {
            sum -= (double)p->lower_ld[(size_t)(d - 1) * w + (size_t)i]
                * out[(ptrdiff_t)(i - d) * os];
        }
        out[(ptrdiff_t)i * os] = sum * (double)p->inverse_diagonal[i];
    }
    for (int32_t i = n - 2; i >= 0; --i) {
        double sum = 0.0;
        for (int32_t d = imin(hb, n - i - 1); d >= 1; --d) {
            sum += (double)p->upper_l[(size_t)(d - 1) * w + (size_t)i]
                * out[(ptrdiff_t)(i + d) * os];
        }
        out[(ptrdiff_t)i * os] -= sum;
    }
}

/* inverse_axis_f32 (:1409-1449): Float64 plans run in double with a
 * non-finite check on the way in and out. */
int orc_inverse_axis_f32(const orc_plan *p, const float *in, ptrdiff_t is,
                         float *out, ptrdiff_t os)
{
    if (!p || !in || !out || is == 0 || os == 0) return ORC_INVALID;
    if (p->has_f64) {
        double *src = malloc((size_t)p->source_size * sizeof(double));
        double *dst = malloc((size_t)p->destination_size * sizeof(double));
        if (!src || !dst) { free(src); free(dst); return ORC_NOMEM; }
        int status = ORC_OK;
        for (int32_t i = 0; i < p->source_size; ++i) {
            float v = in[(ptrdiff_t)i * is];
            if (!isfinite(v)) { status = ORC_RUNTIME; break; }
            src[i] = (double)v;
        }
        if (!status) {
            orc_inverse_axis_f64(p, src, 1, dst, 1);
            for (int32_t i = 0; i < p->destination_size; ++i) {
                const float c = (float)dst[i];
                if (!isfinite(dst[i]) || !isfinite(c)) { status = ORC_RUNTIME; break; }
                out[(ptrdiff_t)i * os] = c;
            }
        }
        free(src);
        free(dst);
        return status;
    }
    inverse_axis_f32_scalar(p, in, is, out, os);
    return ORC_OK;
}

/* detail::inverse_axis_f32_ordered (:1068-1122): the same solve with fused
 * multiply-adds, the reference CUDA kernels' operation order. */
void orc_inverse_axis_f32_ordered(const orc_plan *p, const float *in,
                                  ptrdiff_t is, float *out, ptrdiff_t os)
{
    const int32_t n = p->destination_size, hb = p->half_bandwidth;
    const size_t w = (size_t)n;
    for (int32_t i = 0; i < n; ++i) {
        float v = 0.0f;
        for (uint32_t k = p->transpose_offsets[i]; k < p->transpose_offsets[i + 1]; ++k) {
            v = fmaf(p->transpose_weights[k],
                     in[(ptrdiff_t)p->transpose_indices[k] * is], v);
        }
        for (int32_t d = imin(hb, i); d >= 1; --d) {
            v = fmaf(-p->lower_ld[(size_t)(d - 1) * w + (size_t)i],
                     out[(ptrdiff_t)(i - d) * os], v);
        }
        out[(ptrdiff_t)i * os] = v * p->inverse_diagonal[i];
    }
    for (int32_t i = n - 2; i >= 0; --i) {
        float v = out[(ptrdiff_t)i * os];
        const int32_t avail = imin(hb, n - i - 1);
        if (hb == 3) {
            for (int32_t d = 1; d <= avail; ++d) {
                v = fmaf(-p->upper_l[(size_t)(d - 1) * w + (size_t)i],
                         out[(ptrdiff_t)(i + d) * os], v);
            }
        } else {
            for (int32_t d = avail; d >= 1; --d) {
                v = fmaf(-p->upper_l[(size_t)(d - 1) * w + (size_t)i],
                         out[(ptrdiff_t)(i + d) * os], v);
            }
        }
        out[(ptrdiff_t)i * os] = v;
    }
}

/* detail::inverse_axis_f64_ordered (:1124-1191) */
void orc_inverse_axis_f64_ordered(const orc_plan *p, const double *in,
                                  ptrdiff_t is, double *out, ptrdiff_t os)
{
    const int32_t n = p->destination_size, hb = p->half_bandwidth;
    const size_t w = (size_t)n;
    const int retained = p->has_f64;
    for (int32_t i = 0; i < n; ++i) {
        double v = 0.0;
        for (uint32_t k = p->transpose_offsets[i]; k < p->transpose_offsets[i + 1]; ++k) {
            const double wt = retained ? p->transpose_weights_f64[k]
                                       : (double)p->transpose_weights[k];
            v = fma(wt, in[(ptrdiff_t)p->transpose_indices[k] * is], v);
        }
        for (int32_t d = imin(hb, i); d >= 1; --d) {
            const double f = retained
                ? p->ldlt_bands_f64[(size_t)d * w + (size_t)(i - d)]
                : (double)p->lower_ld[(size_t)(d - 1) * w + (size_t)i];
            v = fma(-f, out[(ptrdiff_t)(i - d) * os], v);
        }
        out[(ptrdiff_t)i * os] = retained
            ? v : v * (double)p->inverse_diagonal[i];
    }
    if (retained) {
        for (int32_t i = 0; i < n; ++i) out[(ptrdiff_t)i * os] *= p->inverse_diagonal_f64[i];
    }
    for (int32_t i = n - 2; i >= 0; --i) {
        double v = out[(ptrdiff_t)i * os];
        for (int32_t d = imin(hb, n - i - 1); d >= 1; --d) {
            const double f = retained
                ? p->ldlt_bands_f64[(size_t)d * w + (size_t)i]
                : (double)p->upper_l[(size_t)(d - 1) * w + (size_t)i];
            v = fma(-f, out[(ptrdiff_t)(i + d) * os], v);
        }
        out[(ptrdiff_t)i * os] = v;
    }
}

/* ---- CpuExecutor(CpuPath::scalar) routes ------------------------------- */

static int plan_ok(const orc_plan *p)
{
    return p && p->source_size > 0 && p->destination_size > 0;
}

/* CpuExecutor::inverse_rows, src/cpu_executor.cpp:903-1172 (scalar branch:
 * inverse_axis_f32 per row; Float64 plans need finite input). */
int orc_inverse_rows(const orc_plan *p, const float *in, ptrdiff_t is,
                     float *out, ptrdiff_t os, int32_t rows)
{
    if (!plan_ok(p) || !in || !out || is < p->source_size
        || os < p->destination_size || rows < 0) return ORC_INVALID;
    if (p->has_f64) {
        for (int32_t r = 0; r < rows; ++r)
            for (int32_t c = 0; c < p->source_size; ++c)
                if (!isfinite(in[(ptrdiff_t)r * is + c])) return ORC_RUNTIME;
    }
    for (int32_t r = 0; r < rows; ++r) {
        int s = orc_inverse_axis_f32(p, in + (ptrdiff_t)r * is, 1,
                                     out + (ptrdiff_t)r * os, 1);
        if (s) return s;
    }
    return ORC_OK;
}

/* CpuExecutor::inverse_columns, src/cpu_executor.cpp:1174-1395 */
int orc_inverse_columns(const orc_plan *p, const float *in, ptrdiff_t is,
                        float *out, ptrdiff_t os, int32_t columns)
{
    if (!plan_ok(p) || !in || !out || columns < 0 || is < columns
        || os < columns) return ORC_INVALID;
    if (p->has_f64) {
        for (int32_t r = 0; r < p->source_size; ++r)
            for (int32_t c = 0; c < columns; ++c)
                if (!isfinite(in[(ptrdiff_t)r * is + c])) return ORC_RUNTIME;
    }
    for (int32_t c = 0; c < columns; ++c) {
        int s = orc_inverse_axis_f32(p, in + c, is, out + c, os);
        if (s) return s;
    }
    return ORC_OK;
}

/* inverse_2d_f64 (src/cpu_executor.cpp:1528-1651): both axes in double when
 * either plan retains Float64.  `kind` 0 = float, 1 = u8, 2 = u16. */
static int inverse_2d_f64(const orc_plan *h, const orc_plan *v,
                          const void *input, ptrdiff_t is, void *output,
                          ptrdiff_t os, const orc_conversion *conv, int kind)
{
    const size_t mid_stride = (size_t)h->destination_size;
    double *mid = malloc((size_t)v->source_size * mid_stride * sizeof(double));
    double *src = malloc((size_t)h->source_size * sizeof(double));
    double *dst = malloc((size_t)v->destination_size * sizeof(double));
    if (!mid || !src || !dst) { free(mid); free(src); free(dst); return ORC_NOMEM; }
    for (int32_t r = 0; r < v->source_size; ++r) {
        for (int32_t c = 0; c < h->source_size; ++c) {
            const ptrdiff_t at = (ptrdiff_t)r * is + c;
            if (kind == 0) {
                src[c] = (double)((const float *)input)[at];
            } else {
                const double sample = kind == 1
                    ? (double)((const uint8_t *)input)[at]
                    : (double)((const uint16_t *)input)[at];
                src[c] = (sample - (double)conv->input_offset)
                    * (double)conv->input_scale;
            }
        }
        orc_inverse_axis_f64(h, src, 1, mid + (size_t)r * mid_stride, 1);
    }
    int nonfinite = 0;
    for (int32_t c = 0; c < h->destination_size; ++c) {
        orc_inverse_axis_f64(v, mid + c, (ptrdiff_t)mid_stride, dst, 1);
        for (int32_t r = 0; r < v->destination_size; ++r) {
            const double value = dst[r];
            const ptrdiff_t at = (ptrdiff_t)r * os + c;
            if (kind == 0) {
                const float f = (float)value;
                if (!isfinite(value) || !isfinite(f)) nonfinite = 1;
                ((float *)output)[at] = f;
            } else {
                const double scaled = value * (double)conv->output_scale
                    + (double)conv->output_offset;
                if (!isfinite(value) || !isfinite(scaled)) {
                    nonfinite = 1;
                    if (kind == 1) ((uint8_t *)output)[at] = 0;
                    else ((uint16_t *)output)[at] = 0;
                    continue;
                }
                const double hi = (double)conv->output_maximum;
                const double cl = scaled < 0.0 ? 0.0 : (scaled > hi ? hi : scaled);
                const double q = nearbyint(cl);
                if (kind == 1) ((uint8_t *)output)[at] = (uint8_t)q;
                else ((uint16_t *)output)[at] = (uint16_t)q;
            }
        }
    }
    free(mid);
    free(src);
    free(dst);
    return nonfinite ? ORC_RUNTIME : ORC_OK;
}

/* CpuExecutor::inverse_2d, src/cpu_executor.cpp:1941-2049.  The scalar
 * Float32 route (forward_2d_rhs_scalar + backward_rhs_scalar) computes every
 * source row's horizontal solve and then one inverse_axis_f32 per column of
 * that intermediate, operation for operation. */
int orc_inverse_2d(const orc_plan *h, const orc_plan *v, const float *in,
                   ptrdiff_t is, float *out, ptrdiff_t os)
{
    if (!plan_ok(h) || !plan_ok(v) || !in || !out || is < h->source_size
        || os < h->destination_size) return ORC_INVALID;
    if (h->has_f64 || v->has_f64) {
        for (int32_t r = 0; r < v->source_size; ++r)
            for (int32_t c = 0; c < h->source_size; ++c)
                if (!isfinite(in[(ptrdiff_t)r * is + c])) return ORC_RUNTIME;
        return inverse_2d_f64(h, v, in, is, out, os, NULL, 0);
    }
    const size_t ms = (size_t)h->destination_size;
    float *mid = malloc((size_t)v->source_size * ms * sizeof(float));
    if (!mid) return ORC_NOMEM;
    for (int32_t r = 0; r < v->source_size; ++r) {
        inverse_axis_f32_scalar(h, in + (ptrdiff_t)r * is, 1, mid + (size_t)r * ms, 1);
    }
    for (int32_t c = 0; c < h->destination_size; ++c) {
        inverse_axis_f32_scalar(v, mid + c, (ptrdiff_t)ms, out + c, os);
    }
    free(mid);
    return ORC_OK;
}

/* CpuExecutor::inverse_2d_integer, src/cpu_executor.cpp:2051-2257 (scalar
 * tail: accumulate_2d_integer_rhs_scalar, solve_rhs_scalar and
 * convert_rhs_to_integer_scalar).  The source-ordered scatter adds the
 * contributions of every destination row in ascending source order, which is
 * the gather order, so it is restated as a gather. */
static int inverse_2d_integer(const orc_plan *h, const orc_plan *v,
                              const void *input, ptrdiff_t is, void *output,
                              ptrdiff_t os, const orc_conversion *conv,
                              int kind)
{
    const uint32_t limit = kind == 1 ? 255U : 65535U;
    if (!plan_ok(h) || !plan_ok(v) || !input || !output || !conv
        || is < h->source_size || os < h->destination_size
        || !(conv->input_scale > 0.0f) || !(conv->output_scale > 0.0f)
        || !isfinite(conv->input_offset) || !isfinite(conv->input_scale)
        || !isfinite(conv->output_scale) || !isfinite(conv->output_offset)
        || conv->output_maximum == 0U || conv->output_maximum > limit) {
        return ORC_INVALID;
    }
    if (h->has_f64 || v->has_f64) {
        return inverse_2d_f64(h, v, input, is, output, os, conv, kind);
    }
    const size_t ms = (size_t)h->destination_size;
    float *mid = malloc((size_t)v->source_size * ms * sizeof(float));
    float *row = malloc((size_t)h->source_size * sizeof(float));
    float *col = malloc((size_t)v->destination_size * sizeof(float));
    if (!mid || !row || !col) { free(mid); free(row); free(col); return ORC_NOMEM; }
    for (int32_t r = 0; r < v->source_size; ++r) {
        for (int32_t c = 0; c < h->source_size; ++c) {
            const ptrdiff_t at = (ptrdiff_t)r * is + c;
            const float sample = kind == 1 ? (float)((const uint8_t *)input)[at]
                                           : (float)((const uint16_t *)input)[at];
            row[c] = (sample - conv->input_offset) * conv->input_scale;
        }
        inverse_axis_f32_scalar(h, row, 1, mid + (size_t)r * ms, 1);
    }
    const float hi = (float)conv->output_maximum;
    for (int32_t c = 0; c < h->destination_size; ++c) {
        inverse_axis_f32_scalar(v, mid + c, (ptrdiff_t)ms, col, 1);
        for (int32_t r = 0; r < v->destination_size; ++r) {
            float scaled = col[r] * conv->output_scale + conv->output_offset;
            scaled = scaled < 0.0f ? 0.0f : (hi < scaled ? hi : scaled);
            const float q = nearbyintf(scaled);
            const ptrdiff_t at = (ptrdiff_t)r * os + c;
            if (kind == 1) ((uint8_t *)output)[at] = (uint8_t)q;
            else ((uint16_t *)output)[at] = (uint16_t)q;
        }
    }
    free(mid);
    free(row);
    free(col);
    return ORC_OK;
}

int orc_inverse_2d_u8(const orc_plan *h, const orc_plan *v,
                      const uint8_t *in, ptrdiff_t is, uint8_t *out,
                      ptrdiff_t os, const orc_conversion *conv)
{
    return inverse_2d_integer(h, v, in, is, out, os, conv, 1);
}

int orc_inverse_2d_u16(const orc_plan *h, const orc_plan *v,
                       const uint16_t *in, ptrdiff_t is, uint16_t *out,
                       ptrdiff_t os, const orc_conversion *conv)
{
    return inverse_2d_integer(h, v, in, is, out, os, conv, 2);
}

/* ---- Reference CUDA operation order ------------------------------------ */

/* The Float32 arithmetic of the reference CUDA kernels
 * (src/cuda/dsmvc_cuda.cu:62-148 inverse_axis_ring and :396-466 solve_axis):
 * the gather is one fmaf chain in CSR order; the forward pass subtracts
 * lower*y with fmaf in descending distance and multiplies by the inverse
 * diagonal; the backward pass accumulates upper*x with fmaf (ascending
 * distance for half-bandwidth 3, descending otherwise) and subtracts the sum
 * once.  The GB300 kernels that solve each vector sequentially follow the
 * same order, so this is their bit-exact expectation. */
void orc_inverse_axis_f32_gpu(const orc_plan *p, const float *in,
                              ptrdiff_t is, float *out, ptrdiff_t os)
{
    const int32_t n = p->destination_size, hb = p->half_bandwidth;
    const size_t w = (size_t)n;
    for (int32_t i = 0; i < n; ++i) {
        float sum = 0.0f;
        for (uint32_t k = p->transpose_offsets[i]; k < p->transpose_offsets[i + 1]; ++k) {
            sum = fmaf(p->transpose_weights[k],
                       in[(ptrdiff_t)p->transpose_indices[k] * is], sum);
        }
        for (int32_t d = imin(hb, i); d >= 1; --d) {
            sum = fmaf(-p->lower_ld[(size_t)(d - 1) * w + (size_t)i],
                       out[(ptrdiff_t)(i - d) * os], sum);
        }
        out[(ptrdiff_t)i * os] = sum * p->inverse_diagonal[i];
    }
    for (int32_t i = n - 2; i >= 0; --i) {
        float sum = 0.0f;
        const int32_t avail = imin(hb, n - i - 1);
        if (hb == 3) {
            for (int32_t d = 1; d <= avail; ++d)
                sum = fmaf(p->upper_l[(size_t)(d - 1) * w + (size_t)i],
                           out[(ptrdiff_t)(i + d) * os], sum);
        } else {
            for (int32_t d = avail; d >= 1; --d)
                sum = fmaf(p->upper_l[(size_t)(d - 1) * w + (size_t)i],
                           out[(ptrdiff_t)(i + d) * os], sum);
        }
        out[(ptrdiff_t)i * os] = out[(ptrdiff_t)i * os] - sum;
    }
}

/* Float32 2D in that order: every source row (with the integer input
 * normalisation (v - offset) * scale), then every column of the
 * intermediate, then the CPU's integer output conversion
 * (src/cpu_executor.cpp:1919-1939).  kind 0 float, 1 u8, 2 u16. */
int orc_inverse_2d_gpu_order(const orc_plan *h, const orc_plan *v, int kind,
                             const void *input, ptrdiff_t is, void *output,
                             ptrdiff_t os, const orc_conversion *conv)
{
    if (!plan_ok(h) || !plan_ok(v) || !input || !output) return ORC_INVALID;
    const size_t ms = (size_t)h->destination_size;
    float *mid = malloc((size_t)v->source_size * ms * sizeof(float));
    float *row = malloc((size_t)h->source_size * sizeof(float));
    float *col = malloc((size_t)v->destination_size * sizeof(float));
    if (!mid || !row || !col) { free(mid); free(row); free(col); return ORC_NOMEM; }
    for (int32_t r = 0; r < v->source_size; ++r) {
        for (int32_t c = 0; c < h->source_size; ++c) {
            const ptrdiff_t at = (ptrdiff_t)r * is + c;
            if (kind == 0) {
                row[c] = ((const float *)input)[at];
            } else {
                const float s = kind == 1 ? (float)((const uint8_t *)input)[at]
                                          : (float)((const uint16_t *)input)[at];
                row[c] = (s - conv->input_offset) * conv->input_scale;
            }
        }
        orc_inverse_axis_f32_gpu(h, row, 1, mid + (size_t)r * ms, 1);
    }
    for (int32_t c = 0; c < h->destination_size; ++c) {
        orc_inverse_axis_f32_gpu(v, mid + c, (ptrdiff_t)ms, col, 1);
        for (int32_t r = 0; r < v->destination_size; ++r) {
            const ptrdiff_t at = (ptrdiff_t)r * os + c;
            if (kind == 0) {
                ((float *)output)[at] = col[r];
                continue;
            }
            const float hi = (float)conv->output_maximum;
            float s = col[r] * conv->output_scale + conv->output_offset;
            s = s < 0.0f ? 0.0f : (hi < s ? hi : s);
            const float q = nearbyintf(s);
            if (kind == 1) ((uint8_t *)output)[at] = (uint8_t)q;
            else ((uint16_t *)output)[at] = (uint16_t)q;
        }
    }
    free(mid);
    free(row);
    free(col);
    return ORC_OK;
}
