/*
 * FP64 CPU oracle for the fpm-rs image-plane FPM hot path.
 *
 * TEST INFRASTRUCTURE ONLY: a complex128 restatement of the reference
 * (hgrecco/fpm-rs 0.2.0-beta.2) used to check the CUDA product path and to
 * time a CPU baseline. The product library never links or calls this file.
 * Each function names the reference file:line it restates. The FFT is our own
 * mixed-radix Cooley-Tukey; the reference uses rustfft 6.4.1, whose values any
 * correct FFT reproduces to rounding (pinned by the round-trip and constant-
 * object known-answer tests of tests/forward_model_tests.rs:12-31,75-101).
 */
#define _GNU_SOURCE
#include "fpm_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
    double re, im;
} cplx;

static inline cplx cx(double re, double im) { cplx z = {re, im}; return z; }
static inline cplx c_add(cplx a, cplx b) { return cx(a.re + b.re, a.im + b.im); }
static inline cplx c_sub(cplx a, cplx b) { return cx(a.re - b.re, a.im - b.im); }
static inline cplx c_mul(cplx a, cplx b) {
    return cx(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re);
}
static inline cplx c_scale(cplx a, double s) { return cx(a.re * s, a.im * s); }
static inline cplx c_conj(cplx a) { return cx(a.re, -a.im); }
static inline double c_norm_sqr(cplx a) { return a.re * a.re + a.im * a.im; }
static inline double c_norm(cplx a) { return hypot(a.re, a.im); }
static inline double c_arg(cplx a) { return atan2(a.im, a.re); }
static inline cplx c_polar(double r, double t) { return cx(r * cos(t), r * sin(t)); }
/* num_complex division (a / b) for a non-zero divisor. */
static inline cplx c_div(cplx a, cplx b) {
    double d = b.re * b.re + b.im * b.im;
    return cx((a.re * b.re + a.im * b.im) / d, (a.im * b.re - a.re * b.im) / d);
}
static inline cplx c_divr(cplx a, double d) { return cx(a.re / d, a.im / d); }

/* ------------------------------------------------------------------ errors */

static __thread char g_error[512];

const char *orc_last_error(void) { return g_error; }

static int32_t fail(int32_t code, const char *fmt, ...) {
    va_list args;
    va_start(args, fmt);
    vsnprintf(g_error, sizeof g_error, fmt, args);
    va_end(args);
    return code;
}

/* --------------------------------------------------------------------- FFT */

/* One cached 1-D plan: forward twiddles e^{-2 pi i t / n} and their exact
 * conjugates for the inverse direction. */
typedef struct {
    int n;
    int pow2;
    cplx *tw;
    cplx *twi;
    int *rev;
} fft_plan;

#define PLAN_CACHE 8
static __thread fft_plan g_plans[PLAN_CACHE];
static __thread int g_plan_next;

static fft_plan *get_plan(int n) {
    for (int i = 0; i < PLAN_CACHE; ++i)
        if (g_plans[i].n == n) return &g_plans[i];
    fft_plan *p = &g_plans[g_plan_next];
    g_plan_next = (g_plan_next + 1) % PLAN_CACHE;
    free(p->tw);
    free(p->twi);
    free(p->rev);
    p->n = n;
    p->tw = (cplx *)malloc(sizeof(cplx) * (size_t)n);
    p->twi = (cplx *)malloc(sizeof(cplx) * (size_t)n);
    for (int t = 0; t < n; ++t) {
        double angle = 2.0 * M_PI * (double)t / (double)n;
        p->tw[t] = cx(cos(angle), -sin(angle));
        p->twi[t] = c_conj(p->tw[t]);
    }
    p->pow2 = (n & (n - 1)) == 0;
    p->rev = NULL;
    if (p->pow2) {
        int bits = 0;
        while ((1 << bits) < n) ++bits;
        p->rev = (int *)malloc(sizeof(int) * (size_t)n);
        for (int i = 0; i < n; ++i) {
            int r = 0;
            for (int b = 0; b < bits; ++b)
                if (i & (1 << b)) r |= 1 << (bits - 1 - b);
            p->rev[i] = r;
        }
    }
    return p;
}

static int smallest_factor(int n) {
    if (n % 2 == 0) return 2;
    for (int f = 3; f * f <= n; f += 2)
        if (n % f == 0) return f;
    return n;
}

/* Two doubles (re, im) as one GCC vector value: portable C (the vector
 * extension, no target intrinsics). Loads and stores go through a type that
 * may sit at 8-byte alignment and may alias the cplx values it reads. */
typedef double v2d __attribute__((vector_size(16)));
typedef double v2d_u __attribute__((vector_size(16), aligned(8), may_alias));

static inline v2d v_load(const cplx *p) { return *(const v2d_u *)p; }
static inline void v_store(cplx *p, v2d v) { *(v2d_u *)p = v; }
/* b * w with w = (wr, wi) and ws = (-wi, wr): (re wr + im (-wi), re wi +
 * im wr), which rounds exactly like c_mul(b, w) since negation is exact. */
static inline v2d v_mul(v2d b, v2d w, v2d ws) {
    v2d re = {b[0], b[0]}, im = {b[1], b[1]};
    return re * w + im * ws;
}

/* Mixed-radix decimation in time over `count` interleaved transforms:
 * out[k] = sum_j in[j istride] w_n^{jk}, where each element is a run of
 * `count` values (one per transform) and out holds element k at k count.
 * The p-point steps of every transform use the same operations in the same
 * order for any count. t and y hold p count values each, for the largest
 * prime p of n; a level uses them only after its sub-transforms return. */
static void dft_multi(const cplx *in, size_t istride, cplx *out, int n, const fft_plan *root, int inverse,
                      size_t count, cplx *t, cplx *y) {
    if (n == 1) {
        memcpy(out, in, sizeof(cplx) * count);
        return;
    }
    int p = smallest_factor(n);
    int m = n / p;
    for (int r = 0; r < p; ++r)
        dft_multi(in + (size_t)r * istride, istride * p, out + (size_t)r * m * count, m, root, inverse, count, t, y);
    int step = root->n / n;
    const cplx *tw = inverse ? root->twi : root->tw;
    for (int k = 0; k < m; ++k) {
        /* Twiddle w_n^{r k}: its exponent (r k mod n) advances by k per r. */
        for (int r = 0, e = 0; r < p; ++r) {
            cplx w = tw[(size_t)e * step];
            v2d wv = {w.re, w.im}, ws = {-w.im, w.re};
            const cplx *src = out + ((size_t)r * m + k) * count;
            cplx *dst = t + (size_t)r * count;
            for (size_t c = 0; c < count; ++c) v_store(dst + c, v_mul(v_load(src + c), wv, ws));
            e += k;
            if (e >= n) e -= n;
        }
        /* The size-p DFT: w_n^{m r q} = w_p^{r q}, exponent (m r q mod n)
         * advancing by m q per r. */
        for (int q = 0; q < p; ++q) {
            cplx *acc = y + (size_t)q * count;
            for (size_t c = 0; c < count; ++c) acc[c] = cx(0.0, 0.0);
            int mq = (int)((long)m * q % n);
            for (int r = 0, e = 0; r < p; ++r) {
                cplx w = tw[(size_t)e * step];
                v2d wv = {w.re, w.im}, ws = {-w.im, w.re};
                const cplx *tr = t + (size_t)r * count;
                for (size_t c = 0; c < count; ++c) v_store(acc + c, v_load(acc + c) + v_mul(v_load(tr + c), wv, ws));
                e += mq;
                if (e >= n) e -= n;
            }
        }
        for (int q = 0; q < p; ++q)
            memcpy(out + ((size_t)k + (size_t)m * q) * count, y + (size_t)q * count, sizeof(cplx) * count);
    }
}

/* Power-of-two radix-2 decimation in time over `count` interleaved
 * transforms: element i of transform c sits at v[i * count + c]. With
 * count = 1 this is one contiguous transform; with count = w it transforms
 * every column of an h x w row-major array at once, each butterfly combining
 * two whole rows, so the inner loop runs over contiguous memory. Every
 * transform sees the same operations in the same order for any count. */
static void fft_pow2(cplx *v, size_t count, const fft_plan *plan, int inverse) {
    int n = plan->n;
    const cplx *tw = inverse ? plan->twi : plan->tw;
    for (int i = 0; i < n; ++i) {
        int r = plan->rev[i];
        if (r <= i) continue;
        cplx *a = v + (size_t)i * count, *b = v + (size_t)r * count;
        for (size_t c = 0; c < count; ++c) {
            cplx tmp = a[c];
            a[c] = b[c];
            b[c] = tmp;
        }
    }
    int len = 2;
    int bits = 0;
    while ((1 << bits) < n) ++bits;
    if (bits & 1) {
        /* One lone stage (butterflies of width 2, twiddle w^0) leaves an
         * even number of stages for the pairs below. */
        v2d w = {tw[0].re, tw[0].im}, ws = {-tw[0].im, tw[0].re};
        for (int start = 0; start < n; start += 2) {
            cplx *a = v + (size_t)start * count, *b = a + count;
            for (size_t c = 0; c < count; ++c) {
                v2d x = v_load(a + c);
                v2d y = v_mul(v_load(b + c), w, ws);
                v_store(a + c, x + y);
                v_store(b + c, x - y);
            }
        }
        len = 4;
    }
    /* Stages len and 2 len together: for j < h = len / 2 the four points
     * start + j + {0, h, 2h, 3h} meet only each other in both stages, so
     * their four radix-2 butterflies run in registers, in the same order and
     * with the same twiddles as two separate passes. */
    for (; len <= n; len <<= 2) {
        int h = len >> 1;
        size_t step1 = (size_t)(n / len), step2 = step1 >> 1;
        for (int start = 0; start < n; start += 2 * len) {
            for (int j = 0; j < h; ++j) {
                cplx t1 = tw[(size_t)j * step1], t2 = tw[(size_t)j * step2], t3 = tw[(size_t)(j + h) * step2];
                v2d w1 = {t1.re, t1.im}, w1s = {-t1.im, t1.re};
                v2d w2 = {t2.re, t2.im}, w2s = {-t2.im, t2.re};
                v2d w3 = {t3.re, t3.im}, w3s = {-t3.im, t3.re};
                cplx *p0 = v + (size_t)(start + j) * count;
                cplx *p1 = p0 + (size_t)h * count, *p2 = p1 + (size_t)h * count, *p3 = p2 + (size_t)h * count;
                for (size_t c = 0; c < count; ++c) {
                    v2d x0 = v_load(p0 + c), x2 = v_load(p2 + c);
                    v2d y1 = v_mul(v_load(p1 + c), w1, w1s), y3 = v_mul(v_load(p3 + c), w1, w1s);
                    v2d a0 = x0 + y1, a1 = x0 - y1;
                    v2d a2 = x2 + y3, a3 = x2 - y3;
                    v2d z2 = v_mul(a2, w2, w2s), z3 = v_mul(a3, w3, w3s);
                    v_store(p0 + c, a0 + z2);
                    v_store(p2 + c, a0 - z2);
                    v_store(p1 + c, a1 + z3);
                    v_store(p3 + c, a1 - z3);
                }
            }
        }
    }
}

static int largest_prime_factor(int n) {
    int largest = 1;
    while (n > 1) {
        int p = smallest_factor(n);
        largest = p;
        n /= p;
    }
    return largest;
}

/* Unnormalised transforms of length n in place over `count` interleaved
 * transforms (element i of transform c at v[i count + c]). */
static void fft_lines(cplx *v, int n, size_t count, int inverse) {
    if (n <= 1 || count == 0) return;
    fft_plan *plan = get_plan(n);
    if (plan->pow2) {
        fft_pow2(v, count, plan, inverse);
        return;
    }
    size_t p = (size_t)largest_prime_factor(n);
    cplx *work = (cplx *)malloc(sizeof(cplx) * count * ((size_t)n + 2 * p));
    memcpy(work, v, sizeof(cplx) * (size_t)n * count);
    dft_multi(work, count, v, n, plan, inverse, count, work + (size_t)n * count, work + ((size_t)n + p) * count);
    free(work);
}

#define ROW_GROUP 8

/* CpuBackend::fft2 (src/backend/cpu.rs:130-175): rows, then columns; the
 * forward transform is normalised by 1/(h*w) and the inverse is not. Rows
 * are transformed ROW_GROUP at a time, interleaved in a scratch slab, and
 * columns all at once, a whole row per element; each row's and column's
 * arithmetic is that of a transform on its own. */
static void fft2_c(cplx *v, int h, int w, int inverse) {
    if (w > 1) {
        cplx *slab = (cplx *)malloc(sizeof(cplx) * (size_t)w * ROW_GROUP);
        for (int r = 0; r < h; r += ROW_GROUP) {
            int g_count = h - r < ROW_GROUP ? h - r : ROW_GROUP;
            const cplx *rows = v + (size_t)r * w;
            for (int i = 0; i < w; ++i)
                for (int g = 0; g < g_count; ++g) slab[(size_t)i * g_count + g] = rows[(size_t)g * w + i];
            fft_lines(slab, w, (size_t)g_count, inverse);
            for (int g = 0; g < g_count; ++g)
                for (int i = 0; i < w; ++i) v[(size_t)(r + g) * w + i] = slab[(size_t)i * g_count + g];
        }
        free(slab);
    }
    fft_lines(v, h, (size_t)w, inverse);
    if (!inverse) {
        double norm = (double)h * (double)w;
        for (size_t i = 0; i < (size_t)h * w; ++i) v[i] = c_divr(v[i], norm);
    }
}

int32_t orc_fft2(double *values, int32_t h, int32_t w, int32_t inverse) {
    if (h <= 0 || w <= 0) return fail(ORC_INVALID_SHAPE, "FFT dimensions must be non-zero");
    fft2_c((cplx *)values, h, w, inverse);
    return ORC_OK;
}

/* shift_copy (src/model/forward.rs:552-569). */
static void shift_copy(const cplx *src, cplx *dst, int h, int w, int rs, int cs) {
    for (int r = 0; r < h; ++r)
        for (int c = 0; c < w; ++c)
            dst[(size_t)((r + rs) % h) * w + (c + cs) % w] = src[(size_t)r * w + c];
}
/* fftshift_copy / ifftshift_copy (src/model/forward.rs:530-550). */
static void fftshift_c(const cplx *s, cplx *d, int h, int w) { shift_copy(s, d, h, w, h / 2, w / 2); }
static void ifftshift_c(const cplx *s, cplx *d, int h, int w) {
    shift_copy(s, d, h, w, (h + 1) / 2, (w + 1) / 2);
}

int32_t orc_fftshift(const double *src, double *dst, int32_t h, int32_t w) {
    fftshift_c((const cplx *)src, (cplx *)dst, h, w);
    return ORC_OK;
}
int32_t orc_ifftshift(const double *src, double *dst, int32_t h, int32_t w) {
    ifftshift_c((const cplx *)src, (cplx *)dst, h, w);
    return ORC_OK;
}

/* ------------------------------------------------------------- geometry */

/* Rust f64::round: half away from zero, like C round(). */

typedef struct {
    long integer;
    double offset;
    long lower, upper;
} grid_shift;

/* checked_grid_shift (src/model/image_plane_fpm.rs:975-1024). */
static int32_t checked_grid_shift(double value, grid_shift *out) {
    if (!isfinite(value)) return fail(ORC_INVALID_MODEL, "illumination shift must be finite");
    double rounded = round(value);
    long integer = (long)rounded;
    double offset = value - rounded;
    double nearest = round(offset);
    out->integer = integer;
    out->offset = offset;
    if (fabs(offset - nearest) <= 1e-12) {
        out->lower = out->upper = integer + (long)nearest;
    } else if (offset > 0.0) {
        out->lower = integer;
        out->upper = integer + 1;
    } else {
        out->lower = integer - 1;
        out->upper = integer;
    }
    return ORC_OK;
}

typedef struct {
    long lower_start, upper_start;
    double lower_weight, upper_weight;
} axis_interp;

/* interpolation_axis (src/model/crop.rs:266-313). */
static int32_t interpolation_axis(long start, long length, long bound, double offset,
                                  axis_interp *out) {
    if (length == 0 || bound == 0 || !isfinite(offset))
        return fail(ORC_INVALID_MODEL, "subpixel crop dimensions and offset must be finite and non-zero");
    double nearest = round(offset);
    double integer_offset, fraction;
    if (fabs(offset - nearest) <= 1e-12) {
        integer_offset = nearest;
        fraction = 0.0;
    } else {
        integer_offset = floor(offset);
        fraction = offset - integer_offset;
    }
    long lower_start = start + (long)integer_offset;
    if (lower_start < 0) return fail(ORC_INVALID_MODEL, "subpixel crop starts outside the grid");
    long lower_end = lower_start + length;
    int needs_upper = fraction > 0.0;
    if (lower_end > bound || (needs_upper && lower_end >= bound))
        return fail(ORC_INVALID_MODEL, "subpixel crop interpolation stencil lies outside the grid");
    out->lower_start = lower_start;
    out->upper_start = lower_start + (needs_upper ? 1 : 0);
    out->lower_weight = 1.0 - fraction;
    out->upper_weight = fraction;
    return ORC_OK;
}

static int offset_is_zero(double r, double c) { return fabs(r) <= 1e-12 && fabs(c) <= 1e-12; }

/* FourierCrop::extract_subpixel_standard (src/model/crop.rs:129-167), with
 * the integer path extract_standard (:79-102). */
static int32_t extract_patch_c(const cplx *src, int mh, int mw, long sr, long sc, int h, int w,
                               double orow, double ocol, cplx *dst) {
    if (offset_is_zero(orow, ocol)) {
        if (sr < 0 || sc < 0 || sr + h > mh || sc + w > mw)
            return fail(ORC_INVALID_MODEL, "crop lies outside reconstruction shape");
        for (int r = 0; r < h; ++r)
            memcpy(dst + (size_t)r * w, src + (size_t)(sr + r) * mw + sc, sizeof(cplx) * (size_t)w);
        return ORC_OK;
    }
    axis_interp rows, cols;
    int32_t st = interpolation_axis(sr, h, mh, orow, &rows);
    if (st) return st;
    st = interpolation_axis(sc, w, mw, ocol, &cols);
    if (st) return st;
    for (int r = 0; r < h; ++r) {
        long lr = rows.lower_start + r, ur = rows.upper_start + r;
        for (int c = 0; c < w; ++c) {
            long lc = cols.lower_start + c, uc = cols.upper_start + c;
            cplx v = c_scale(src[lr * mw + lc], rows.lower_weight * cols.lower_weight);
            v = c_add(v, c_scale(src[lr * mw + uc], rows.lower_weight * cols.upper_weight));
            v = c_add(v, c_scale(src[ur * mw + lc], rows.upper_weight * cols.lower_weight));
            v = c_add(v, c_scale(src[ur * mw + uc], rows.upper_weight * cols.upper_weight));
            dst[(size_t)r * w + c] = v;
        }
    }
    return ORC_OK;
}

/* FourierCrop::insert_subpixel_adjoint_slice (src/model/crop.rs:188-255). */
static int32_t insert_adjoint_c(cplx *dst, int mh, int mw, long sr, long sc, int h, int w,
                                double orow, double ocol, const cplx *update, double scale) {
    if (!isfinite(scale)) return fail(ORC_INVALID_PARAMETER, "scale must be finite");
    if (offset_is_zero(orow, ocol)) {
        if (sr < 0 || sc < 0 || sr + h > mh || sc + w > mw)
            return fail(ORC_INVALID_MODEL, "crop lies outside reconstruction shape");
        for (int r = 0; r < h; ++r)
            for (int c = 0; c < w; ++c) {
                cplx *o = &dst[(size_t)(sr + r) * mw + sc + c];
                *o = c_add(*o, c_scale(update[(size_t)r * w + c], scale));
            }
        return ORC_OK;
    }
    axis_interp rows, cols;
    int32_t st = interpolation_axis(sr, h, mh, orow, &rows);
    if (st) return st;
    st = interpolation_axis(sc, w, mw, ocol, &cols);
    if (st) return st;
    for (int r = 0; r < h; ++r) {
        long lr = rows.lower_start + r, ur = rows.upper_start + r;
        for (int c = 0; c < w; ++c) {
            long lc = cols.lower_start + c, uc = cols.upper_start + c;
            cplx value = c_scale(update[(size_t)r * w + c], scale);
            cplx *o;
            o = &dst[lr * mw + lc];
            *o = c_add(*o, c_scale(value, rows.lower_weight * cols.lower_weight));
            o = &dst[lr * mw + uc];
            *o = c_add(*o, c_scale(value, rows.lower_weight * cols.upper_weight));
            o = &dst[ur * mw + lc];
            *o = c_add(*o, c_scale(value, rows.upper_weight * cols.lower_weight));
            o = &dst[ur * mw + uc];
            *o = c_add(*o, c_scale(value, rows.upper_weight * cols.upper_weight));
        }
    }
    return ORC_OK;
}

int32_t orc_extract_patch(const double *spectrum, int32_t mh, int32_t mw, int64_t start_row,
                          int64_t start_col, int32_t h, int32_t w, double off_row, double off_col,
                          double *patch) {
    return extract_patch_c((const cplx *)spectrum, mh, mw, (long)start_row, (long)start_col, h, w,
                           off_row, off_col, (cplx *)patch);
}

int32_t orc_insert_adjoint(double *spectrum, int32_t mh, int32_t mw, int64_t start_row,
                           int64_t start_col, int32_t h, int32_t w, double off_row, double off_col,
                           const double *update, double scale) {
    return insert_adjoint_c((cplx *)spectrum, mh, mw, (long)start_row, (long)start_col, h, w,
                            off_row, off_col, (const cplx *)update, scale);
}

/* Optics::validate (src/experiment/optics.rs:128-189). */
static int32_t validate_optics(const orc_optics *o) {
    const double values[6] = {o->wavelength_vacuum_m, o->objective_na, o->magnification,
                              o->camera_pixel_size, o->illumination_refractive_index,
                              o->objective_medium_refractive_index};
    for (int i = 0; i < 6; ++i)
        if (!isfinite(values[i]) || values[i] <= 0.0)
            return fail(ORC_INVALID_PARAMETER, "optics parameters must be finite and positive");
    if (o->objective_na > o->objective_medium_refractive_index)
        return fail(ORC_INVALID_PARAMETER, "objective_na cannot exceed the medium refractive index");
    double pixel = o->camera_pixel_size / o->magnification;
    double limit = o->wavelength_vacuum_m / (2.0 * o->objective_na);
    if (!(pixel < limit))
        return fail(ORC_INVALID_PARAMETER, "camera_pixel_size / magnification violates coherent sampling");
    if (o->has_defocus && !isfinite(o->defocus_distance))
        return fail(ORC_INVALID_PARAMETER, "defocus_distance must be finite");
    return ORC_OK;
}

/* PlanarLedArray::resolve (src/experiment/led_array.rs:292-313) with
 * ArrayPose::transform_point (:87-112) and ResolvedSources::from_positions
 * (src/experiment/illumination.rs:385-421). */
int32_t orc_planar_kvectors(const orc_optics *optics, int32_t rows, int32_t cols, double pitch_x,
                            double pitch_y, double ref_col, double ref_row,
                            const double *translation, const double *rotation, double *kx,
                            double *ky) {
    int32_t st = validate_optics(optics);
    if (st) return st;
    double k = 2.0 * M_PI * optics->illumination_refractive_index / optics->wavelength_vacuum_m;
    double sx = sin(rotation[0]), cxr = cos(rotation[0]);
    double sy = sin(rotation[1]), cyr = cos(rotation[1]);
    double sz = sin(rotation[2]), czr = cos(rotation[2]);
    for (int r = 0; r < rows; ++r)
        for (int c = 0; c < cols; ++c) {
            double p[3] = {((double)c - ref_col) * pitch_x, ((double)r - ref_row) * pitch_y, 0.0};
            double ax[3] = {p[0], cxr * p[1] - sx * p[2], sx * p[1] + cxr * p[2]};
            double ay[3] = {cyr * ax[0] + sy * ax[2], ax[1], -sy * ax[0] + cyr * ax[2]};
            double rz[3] = {czr * ay[0] - sz * ay[1], sz * ay[0] + czr * ay[1], ay[2]};
            double pos[3] = {rz[0] + translation[0], rz[1] + translation[1], rz[2] + translation[2]};
            double norm = hypot(hypot(pos[0], pos[1]), pos[2]);
            if (!isfinite(norm) || norm <= 0.0)
                return fail(ORC_INVALID_PARAMETER, "no source may coincide with the sample origin");
            int i = r * cols + c;
            kx[i] = k * (-pos[0] / norm);
            ky[i] = k * (-pos[1] / norm);
        }
    return ORC_OK;
}

typedef struct {
    long min_row, max_row, min_col, max_col;
} disp_bounds;

/* crop_displacement_bounds (src/model/image_plane_fpm.rs:255-285). */
static int32_t displacement_bounds(const orc_optics *o, int n, const double *kx, const double *ky,
                                   int h, int w, disp_bounds *b) {
    if (h <= 0 || w <= 0) return fail(ORC_INVALID_SHAPE, "image shape must be non-zero");
    if (n <= 0) return fail(ORC_INVALID_MODEL, "illumination must contain at least one frame");
    double pixel = o->camera_pixel_size / o->magnification;
    double dkx = 2.0 * M_PI / ((double)w * pixel);
    double dky = 2.0 * M_PI / ((double)h * pixel);
    b->min_row = b->min_col = 0x7fffffffffffffffL;
    b->max_row = b->max_col = -0x7fffffffffffffffL - 1;
    for (int i = 0; i < n; ++i) {
        grid_shift row = {0, 0.0, 0, 0}, col = {0, 0.0, 0, 0};
        int32_t st = checked_grid_shift(ky[i] / dky, &row);
        if (st) return st;
        st = checked_grid_shift(kx[i] / dkx, &col);
        if (st) return st;
        if (row.lower < b->min_row) b->min_row = row.lower;
        if (row.upper > b->max_row) b->max_row = row.upper;
        if (col.lower < b->min_col) b->min_col = col.lower;
        if (col.upper > b->max_col) b->max_col = col.upper;
    }
    return ORC_OK;
}

/* axis_contains_bounds (src/model/image_plane_fpm.rs:1089-1114). */
static int axis_contains(long len, long recon, long lo, long hi) {
    long base = recon / 2 - len / 2;
    long lower = base + lo;
    long upper = base + (len - 1) + hi;
    return lower >= 0 && upper < recon;
}

static int shape_fits(int h, int w, long mh, long mw, const disp_bounds *b) {
    return axis_contains(h, mh, b->min_row, b->max_row) && axis_contains(w, mw, b->min_col, b->max_col);
}

static long gcd_l(long a, long b) {
    while (b != 0) {
        long t = a % b;
        a = b;
        b = t;
    }
    return a;
}

/* next_smooth_multiplier (src/model/image_plane_fpm.rs:1176-1198). */
static void smooth_visit(long value, int prime_index, long minimum, long *best) {
    static const long primes[4] = {2, 3, 5, 7};
    if (value >= minimum) {
        if (*best < 0 || value < *best) *best = value;
        return;
    }
    for (int i = prime_index; i < 4; ++i) {
        long next = value * primes[i];
        if (*best < 0 || next < *best) smooth_visit(next, i, minimum, best);
    }
}

int32_t orc_next_smooth(int64_t minimum, int64_t *out) {
    long best = -1;
    smooth_visit(1, 0, (long)minimum, &best);
    *out = best;
    return ORC_OK;
}

/* resolve_reconstruction_shape (src/model/image_plane_fpm.rs:287-348) with
 * minimum_fitting_multiplier (:1116-1155). */
static int32_t resolve_shape(int h, int w, int policy, int emh, int emw, const disp_bounds *b,
                             int32_t *mh, int32_t *mw) {
    if (policy == ORC_SHAPE_EXACT) {
        if (emh < h || emw < w)
            return fail(ORC_INVALID_SHAPE, "image shape must fit reconstruction shape");
        if ((long)emh * w != (long)emw * h)
            return fail(ORC_INVALID_SHAPE, "reconstruction must use the same scale factor in both dimensions");
        if (!shape_fits(h, w, emh, emw, b))
            return fail(ORC_INVALID_SHAPE,
                        "reconstruction shape does not contain every illumination crop and subpixel interpolation stencil");
        *mh = emh;
        *mw = emw;
        return ORC_OK;
    }
    long d = gcd_l(h, w);
    long ah = h / d, aw = w / d;
    long maximum = 1L << 40;
    long multiplier;
    if (shape_fits(h, w, ah * d, aw * d, b)) {
        multiplier = d;
    } else {
        long lower = d, upper = d;
        for (;;) {
            long doubled = upper * 2;
            upper = doubled < maximum ? doubled : maximum;
            if (upper == lower)
                return fail(ORC_INVALID_SHAPE, "illumination crops require a reconstruction shape outside the supported range");
            if (shape_fits(h, w, ah * upper, aw * upper, b)) break;
            lower = upper;
        }
        while (lower + 1 < upper) {
            long middle = lower + (upper - lower) / 2;
            if (shape_fits(h, w, ah * middle, aw * middle, b))
                upper = middle;
            else
                lower = middle;
        }
        multiplier = upper;
    }
    if (policy == ORC_SHAPE_SMOOTH) {
        long best = -1;
        smooth_visit(1, 0, multiplier, &best);
        multiplier = best;
    } else if (policy == ORC_SHAPE_POW2) {
        long p = 1;
        while (p < multiplier) p <<= 1;
        multiplier = p;
    }
    *mh = (int32_t)(ah * multiplier);
    *mw = (int32_t)(aw * multiplier);
    return ORC_OK;
}

int32_t orc_suggest_shape(const orc_optics *optics, int32_t sources, const double *kx,
                          const double *ky, int32_t h, int32_t w, int32_t policy, int32_t *mh,
                          int32_t *mw) {
    int32_t st = validate_optics(optics);
    if (st) return st;
    disp_bounds b;
    st = displacement_bounds(optics, sources, kx, ky, h, w, &b);
    if (st) return st;
    return resolve_shape(h, w, policy, *mh, *mw, &b, mh, mw);
}

/* ImagePlaneModel::compile (src/model/image_plane_fpm.rs:196-253),
 * crop_for_k_vector (:750-797) and Pupil::circular (src/model/pupil.rs:78-123). */
int32_t orc_compile(const orc_optics *optics, int32_t sources, const double *kx, const double *ky,
                    int32_t h, int32_t w, int32_t policy, int32_t exact_mh, int32_t exact_mw,
                    orc_compiled *out) {
    int32_t st = validate_optics(optics);
    if (st) return st;
    disp_bounds b;
    st = displacement_bounds(optics, sources, kx, ky, h, w, &b);
    if (st) return st;
    int32_t mh, mw;
    st = resolve_shape(h, w, policy, exact_mh, exact_mw, &b, &mh, &mw);
    if (st) return st;
    double scale = (double)mw / (double)w;
    double low = optics->camera_pixel_size / optics->magnification;
    out->h = h;
    out->w = w;
    out->mh = mh;
    out->mw = mw;
    out->sources = sources;
    out->low_res_pixel_size = low;
    out->high_res_pixel_size = low / scale;
    out->dkx = 2.0 * M_PI / ((double)w * low);
    out->dky = 2.0 * M_PI / ((double)h * low);
    double cutoff = 2.0 * M_PI * optics->objective_na / optics->wavelength_vacuum_m;
    double medium_k = 2.0 * M_PI * optics->objective_medium_refractive_index / optics->wavelength_vacuum_m;
    cplx *pupil = (cplx *)out->pupil;
    for (int r = 0; r < h; ++r) {
        double y = ((double)r - (double)(h / 2)) * out->dky;
        for (int c = 0; c < w; ++c) {
            double x = ((double)c - (double)(w / 2)) * out->dkx;
            double radius = hypot(x, y);
            int inside = radius <= cutoff;
            size_t i = (size_t)r * w + c;
            out->support[i] = (uint8_t)inside;
            if (!inside) {
                pupil[i] = cx(0.0, 0.0);
                continue;
            }
            double rho = cutoff > 0.0 ? radius / cutoff : 0.0;
            double theta = atan2(y, x);
            double phase = 0.0;
            if (optics->has_defocus) phase -= optics->defocus_distance * (x * x + y * y) / (2.0 * medium_k);
            double amplitude = 1.0;
            if (optics->has_aberration) {
                phase += optics->astigmatism * rho * rho * cos(2.0 * theta);
                phase += optics->coma * (3.0 * pow(rho, 3) - 2.0 * rho) * cos(theta);
                phase += optics->spherical * (6.0 * pow(rho, 4) - 6.0 * rho * rho + 1.0);
                amplitude = exp(-optics->edge_apodization * rho * rho);
            }
            pupil[i] = c_polar(amplitude, phase);
        }
    }
    long center_row = mh / 2, center_col = mw / 2;
    for (int s = 0; s < sources; ++s) {
        grid_shift row = {0, 0.0, 0, 0}, col = {0, 0.0, 0, 0};
        st = checked_grid_shift(ky[s] / out->dky, &row);
        if (st) return st;
        st = checked_grid_shift(kx[s] / out->dkx, &col);
        if (st) return st;
        long start_row = center_row - h / 2 + row.integer;
        long start_col = center_col - w / 2 + col.integer;
        if (start_row < 0 || start_col < 0)
            return fail(ORC_INVALID_MODEL, "illumination vector produces a crop outside the reconstruction grid");
        axis_interp ai;
        st = interpolation_axis(start_row, h, mh, row.offset, &ai);
        if (st) return st;
        st = interpolation_axis(start_col, w, mw, col.offset, &ai);
        if (st) return st;
        out->start_row[s] = start_row;
        out->start_col[s] = start_col;
        out->off_row[s] = row.offset;
        out->off_col[s] = col.offset;
    }
    return ORC_OK;
}

/* ---------------------------------------------------------------- losses */

/* point_loss (src/algorithms/objective.rs:47-71). */
static double point_loss(double predicted, double measured, int loss) {
    switch (loss) {
    case ORC_LOSS_AMPLITUDE_MSE: {
        double r = sqrt(fmax(predicted, 0.0)) - sqrt(fmax(measured, 0.0));
        return r * r;
    }
    case ORC_LOSS_INTENSITY_MSE: {
        double r = predicted - measured;
        return r * r;
    }
    case ORC_LOSS_POISSON_NLL: {
        double mean = fmax(predicted, 1e-12);
        return mean - fmax(measured, 0.0) * log(mean);
    }
    default: {
        double r = sqrt(fmax(predicted, 0.0)) - sqrt(fmax(measured, 0.0));
        double a = fabs(r);
        return a <= 1.0 ? 0.5 * r * r : a - 0.5;
    }
    }
}

/* descent_factor (src/algorithms/gradient_descent.rs:1167-1178). */
static double descent_factor(double predicted, double measured, int loss, double epsilon) {
    switch (loss) {
    case ORC_LOSS_AMPLITUDE_MSE:
        return 1.0 - sqrt(fmax(measured, 0.0)) / sqrt(fmax(predicted, epsilon));
    case ORC_LOSS_INTENSITY_MSE:
        return 2.0 * (predicted - measured);
    case ORC_LOSS_POISSON_NLL:
        return 1.0 - fmax(measured, 0.0) / fmax(predicted, epsilon);
    default: {
        double pa = sqrt(fmax(predicted, epsilon));
        double r = pa - sqrt(fmax(measured, 0.0));
        if (r < -1.0) r = -1.0;
        if (r > 1.0) r = 1.0;
        return r / (2.0 * pa);
    }
    }
}

/* ------------------------------------------------------------------ state */

typedef struct {
    const orc_problem *p;
    int h, w, mh, mw, frames;
    size_t n_low, n_high;
    cplx *object;   /* centred spectrum */
    cplx *pupil;
    double *gains;  /* frames */
    double *background; /* NULL or frames*n_low (expanded) */
    cplx *velocity, *anchor;
    long momentum_count;
    /* scratch */
    cplx *patch, *exit_spec, *field, *projected, *difference, *spectrum, *pupil_gradient, *gradient;
    double *prediction;
    /* GD illumination recovery: per-source (row, column) offset corrections,
     * per-source (gradient row, column, curvature row, column, weight) of the
     * batch, and per-frame scratch. NULL when off. */
    double *corr, *ill, *calref, *fd_plus, *fd_minus;
    uint8_t *dgmask;
    cplx *fd_patch, *fd_field;
} orc_state;

static double frame_weight(const orc_problem *p, int f) { return p->weights ? p->weights[f] : 1.0; }
static const uint8_t *frame_mask(const orc_problem *p, int f) {
    return p->masks ? p->masks + (size_t)f * p->h * p->w : NULL;
}
static double model_gain(const orc_problem *p, int f) { return p->gains ? p->gains[f] : 1.0; }
static double model_background(const orc_problem *p, int f, size_t pixel) {
    if (!p->background) return 0.0;
    size_t n = (size_t)p->h * p->w;
    return p->background_len == (int64_t)n ? p->background[pixel] : p->background[(size_t)f * n + pixel];
}
static double state_background(const orc_state *s, int f, size_t pixel) {
    return s->background ? s->background[(size_t)f * s->n_low + pixel] : 0.0;
}

static void state_free(orc_state *s) {
    free(s->object);
    free(s->pupil);
    free(s->gains);
    free(s->background);
    free(s->velocity);
    free(s->anchor);
    free(s->patch);
    free(s->exit_spec);
    free(s->field);
    free(s->projected);
    free(s->difference);
    free(s->spectrum);
    free(s->pupil_gradient);
    free(s->gradient);
    free(s->prediction);
    free(s->corr);
    free(s->ill);
    free(s->calref);
    free(s->fd_plus);
    free(s->fd_minus);
    free(s->dgmask);
    free(s->fd_patch);
    free(s->fd_field);
}

static void illumination_alloc(orc_state *s) {
    s->corr = (double *)calloc(2 * (size_t)s->frames, sizeof(double));
    s->ill = (double *)calloc(5 * (size_t)s->frames, sizeof(double));
    s->calref = (double *)calloc(s->n_low, sizeof(double));
    s->fd_plus = (double *)calloc(s->n_low, sizeof(double));
    s->fd_minus = (double *)calloc(s->n_low, sizeof(double));
    s->dgmask = (uint8_t *)calloc(s->n_low, 1);
    s->fd_patch = (cplx *)calloc(s->n_low, sizeof(cplx));
    s->fd_field = (cplx *)calloc(s->n_low, sizeof(cplx));
}

/* ReconstructionProblem::validate (src/reconstruction/problem.rs:35-72) and
 * MeasurementStack::validate (src/measurements/stack.rs:377-...). */
static int32_t validate_problem(const orc_problem *p) {
    size_t n = (size_t)p->h * p->w;
    if (p->h <= 0 || p->w <= 0 || p->frames <= 0)
        return fail(ORC_INVALID_MEASUREMENTS, "stored frame count, image shape, and data length are inconsistent");
    for (size_t i = 0; i < n * p->frames; ++i)
        if (!isfinite(p->data[i])) return fail(ORC_INVALID_MEASUREMENTS, "measurements contain non-finite values");
    int positive = 0;
    for (int f = 0; f < p->frames; ++f) {
        double wgt = frame_weight(p, f);
        if (!isfinite(wgt) || wgt < 0.0) return fail(ORC_INVALID_MEASUREMENTS, "frame %d has invalid weight", f);
        if (wgt > 0.0) {
            ++positive;
            const uint8_t *m = frame_mask(p, f);
            if (m) {
                int any = 0;
                for (size_t i = 0; i < n; ++i) any |= m[i] != 0;
                if (!any) return fail(ORC_INVALID_MEASUREMENTS, "positive-weight frame %d has no unmasked pixels", f);
            }
        }
        double g = model_gain(p, f);
        if (!isfinite(g) || g < 0.0) return fail(ORC_INVALID_MODEL, "frame gains must be finite and non-negative");
    }
    if (positive == 0) return fail(ORC_INVALID_MEASUREMENTS, "at least one frame must have positive weight");
    return ORC_OK;
}

/* ReconstructionState::initialize_with_backend (src/reconstruction/state.rs:280-355). */
static int32_t state_init(orc_state *s, const orc_problem *p) {
    memset(s, 0, sizeof *s);
    s->p = p;
    s->h = p->h;
    s->w = p->w;
    s->mh = p->mh;
    s->mw = p->mw;
    s->frames = p->frames;
    s->n_low = (size_t)p->h * p->w;
    s->n_high = (size_t)p->mh * p->mw;
    int32_t st = validate_problem(p);
    if (st) return st;
    double *average = (double *)calloc(s->n_low, sizeof(double));
    double *weight = (double *)calloc(s->n_low, sizeof(double));
    double total_amplitude = 0.0, total_weight = 0.0;
    for (int f = 0; f < p->frames; ++f) {
        double fw = frame_weight(p, f);
        if (fw == 0.0) continue;
        const uint8_t *mask = frame_mask(p, f);
        double gain = model_gain(p, f);
        const double *frame = p->data + (size_t)f * s->n_low;
        for (size_t i = 0; i < s->n_low; ++i) {
            if (mask && mask[i] == 0) continue;
            double amplitude = sqrt(fmax((frame[i] - model_background(p, f, i)) / gain, 0.0));
            average[i] += fw * amplitude;
            weight[i] += fw;
            total_amplitude += fw * amplitude;
            total_weight += fw;
        }
    }
    if (total_weight == 0.0) {
        free(average);
        free(weight);
        return fail(ORC_INVALID_MEASUREMENTS, "no positive-weight, unmasked measurements are available");
    }
    double fallback = total_amplitude / total_weight;
    for (size_t i = 0; i < s->n_low; ++i) average[i] = weight[i] > 0.0 ? average[i] / weight[i] : fallback;
    cplx *object = (cplx *)malloc(sizeof(cplx) * s->n_high);
    for (int r = 0; r < s->mh; ++r) {
        long lr = (long)r * s->h / s->mh;
        for (int c = 0; c < s->mw; ++c) {
            long lc = (long)c * s->w / s->mw;
            object[(size_t)r * s->mw + c] = cx(average[lr * s->w + lc], 0.0);
        }
    }
    free(average);
    free(weight);
    fft2_c(object, s->mh, s->mw, 0);
    s->object = (cplx *)malloc(sizeof(cplx) * s->n_high);
    fftshift_c(object, s->object, s->mh, s->mw);
    free(object);
    s->pupil = (cplx *)malloc(sizeof(cplx) * s->n_low);
    memcpy(s->pupil, p->pupil, sizeof(cplx) * s->n_low);
    s->gains = (double *)malloc(sizeof(double) * (size_t)p->frames);
    for (int f = 0; f < p->frames; ++f) s->gains[f] = model_gain(p, f);
    if (p->background) {
        s->background = (double *)malloc(sizeof(double) * s->n_low * p->frames);
        for (int f = 0; f < p->frames; ++f)
            for (size_t i = 0; i < s->n_low; ++i) s->background[(size_t)f * s->n_low + i] = model_background(p, f, i);
    }
    s->patch = (cplx *)malloc(sizeof(cplx) * s->n_low);
    s->exit_spec = (cplx *)malloc(sizeof(cplx) * s->n_low);
    s->field = (cplx *)malloc(sizeof(cplx) * s->n_low);
    s->projected = (cplx *)malloc(sizeof(cplx) * s->n_low);
    s->difference = (cplx *)malloc(sizeof(cplx) * s->n_low);
    s->spectrum = (cplx *)malloc(sizeof(cplx) * s->n_low);
    s->pupil_gradient = (cplx *)calloc(s->n_low, sizeof(cplx));
    s->prediction = (double *)malloc(sizeof(double) * s->n_low);
    return ORC_OK;
}

static double src_off_row(const orc_problem *p, int s) { return p->off_row ? p->off_row[s] : 0.0; }
static double src_off_col(const orc_problem *p, int s) { return p->off_col ? p->off_col[s] : 0.0; }
/* ReconstructionState::effective_source_offset (src/reconstruction/state.rs:
 * 245-267): the compiled offset plus the recovered illumination correction. */
static double eff_off_row(const orc_state *s, int src) {
    return src_off_row(s->p, src) + (s->corr ? s->corr[2 * src] : 0.0);
}
static double eff_off_col(const orc_state *s, int src) {
    return src_off_col(s->p, src) + (s->corr ? s->corr[2 * src + 1] : 0.0);
}

/* Patch, pupil, ifftshift and inverse FFT: the coherent detector field of one
 * source (src/algorithms/common.rs:94-131, gradient_descent.rs:1184-1213). */
static int32_t source_field(orc_state *s, int source) {
    const orc_problem *p = s->p;
    int32_t st = extract_patch_c(s->object, s->mh, s->mw, (long)p->start_row[source], (long)p->start_col[source],
                                 s->h, s->w, eff_off_row(s, source), eff_off_col(s, source), s->patch);
    if (st) return st;
    for (size_t i = 0; i < s->n_low; ++i) s->exit_spec[i] = c_mul(s->patch[i], s->pupil[i]);
    ifftshift_c(s->exit_spec, s->field, s->h, s->w);
    fft2_c(s->field, s->h, s->w, 1);
    return ORC_OK;
}

typedef struct {
    double object_step, epsilon;
    int loss;
    int denominator; /* 0 local, 1 rpie, 2 global */
    double alpha;
    int has_pupil_step;
    double pupil_step;
    int constrain_pupil;
    int gain_update;
    double gain_step, gain_min, gain_max;
    int background_update;
    double background_step, background_min, background_max;
    int momentum;
    long interval;
    double friction, feedback;
} update_config;

typedef struct {
    double objective_sum, weight_sum;
} step_summary;

/* apply_momentum_event (src/algorithms/common.rs:355-387). */
int32_t orc_momentum_event(double *object_d, double *velocity_d, double *anchor_d, int64_t len,
                           double friction, double feedback) {
    cplx *object = (cplx *)object_d, *velocity = (cplx *)velocity_d, *anchor = (cplx *)anchor_d;
    for (int64_t i = 0; i < len; ++i) {
        cplx nv = c_add(c_scale(velocity[i], friction), c_sub(object[i], anchor[i]));
        cplx no = feedback == 0.0 ? object[i] : c_add(object[i], c_scale(nv, feedback));
        if (!isfinite(nv.re) || !isfinite(nv.im) || !isfinite(no.re) || !isfinite(no.im))
            return fail(ORC_NUMERICAL, "mPIE momentum produced a non-finite object or velocity");
        velocity[i] = nv;
        object[i] = no;
        anchor[i] = no;
    }
    return ORC_OK;
}

/* projection_update (src/algorithms/common.rs:57-306) for non-multiplexed
 * frames, with update_gain (:390-422), update_background (:425-489) and
 * apply_object_momentum (:308-353). */
static int32_t projection_update(orc_state *s, const int *frames, int count, const update_config *cfg,
                                 step_summary *summary) {
    const orc_problem *p = s->p;
    size_t n = s->n_low;
    for (int b = 0; b < count; ++b) {
        int frame = frames[b];
        double fw = frame_weight(p, frame);
        if (fw == 0.0) continue;
        double source_weight_sum = 1.0;
        int32_t st = source_field(s, frame);
        if (st) return st;
        for (size_t i = 0; i < n; ++i) s->prediction[i] = c_norm_sqr(s->field[i]);
        const double *measured = p->data + (size_t)frame * n;
        const uint8_t *mask = frame_mask(p, frame);
        double gain = s->gains[frame];
        if (!isfinite(gain) || gain <= 0.0) return fail(ORC_INVALID_MODEL, "state frame %d has invalid gain", frame);
        if (cfg->gain_update) {
            double num = 0.0, den = 0.0;
            for (size_t i = 0; i < n; ++i) {
                if (mask && mask[i] == 0) continue;
                double pred = s->prediction[i];
                num += pred * fmax(measured[i] - state_background(s, frame, i), 0.0);
                den += pred * pred;
            }
            if (den > cfg->epsilon) {
                double est = fmin(fmax(num / den, cfg->gain_min), cfg->gain_max);
                gain = fmin(fmax((1.0 - cfg->gain_step) * gain + cfg->gain_step * est, cfg->gain_min), cfg->gain_max);
                s->gains[frame] = gain;
            }
        }
        if (cfg->background_update) {
            double residual = 0.0;
            long rc = 0;
            for (size_t i = 0; i < n; ++i) {
                if (mask && mask[i] == 0) continue;
                residual += measured[i] - gain * s->prediction[i] - state_background(s, frame, i);
                ++rc;
            }
            if (rc > 0) {
                double correction = cfg->background_step * residual / (double)rc;
                if (!s->background) s->background = (double *)calloc(n * s->frames, sizeof(double));
                double *bg = s->background + (size_t)frame * n;
                for (size_t i = 0; i < n; ++i)
                    bg[i] = fmin(fmax(bg[i] + correction, cfg->background_min), cfg->background_max);
            }
        }
        double frame_loss = 0.0;
        long valid = 0;
        for (size_t i = 0; i < n; ++i) {
            double intrinsic = s->prediction[i];
            if (mask && mask[i] == 0) {
                s->projected[i] = cx(1.0, 0.0);
                continue;
            }
            ++valid;
            double bg = state_background(s, frame, i);
            double predicted = gain * intrinsic + bg;
            frame_loss += point_loss(predicted, measured[i], cfg->loss);
            double target = fmax((measured[i] - bg) / gain, 0.0);
            s->projected[i] = intrinsic > cfg->epsilon ? cx(sqrt(target / intrinsic), 0.0)
                                                       : cx(0.0, sqrt(target / source_weight_sum));
        }
        if (valid == 0) return fail(ORC_INVALID_MEASUREMENTS, "frame %d has no unmasked pixels", frame);
        summary->objective_sum += fw * (frame_loss / (double)valid);
        summary->weight_sum += fw;
        double max_pupil = 0.0;
        for (size_t i = 0; i < n; ++i) max_pupil = fmax(max_pupil, c_norm_sqr(s->pupil[i]));
        max_pupil = fmax(max_pupil, cfg->epsilon);
        if (cfg->has_pupil_step) memset(s->pupil_gradient, 0, sizeof(cplx) * n);
        for (size_t i = 0; i < n; ++i) {
            cplx proj = s->projected[i];
            if (mask && mask[i] == 0)
                s->difference[i] = s->field[i];
            else if (s->prediction[i] > cfg->epsilon)
                s->difference[i] = c_scale(s->field[i], proj.re);
            else
                s->difference[i] = cx(proj.im, 0.0);
        }
        fft2_c(s->difference, s->h, s->w, 0);
        fftshift_c(s->difference, s->spectrum, s->h, s->w);
        for (size_t i = 0; i < n; ++i) s->difference[i] = c_sub(s->spectrum[i], c_mul(s->patch[i], s->pupil[i]));
        double normalized = 1.0 / source_weight_sum;
        for (size_t i = 0; i < n; ++i) {
            cplx pup = s->pupil[i];
            double local = c_norm_sqr(pup);
            double den;
            if (cfg->denominator == 0)
                den = local + cfg->epsilon;
            else if (cfg->denominator == 2)
                den = max_pupil + cfg->epsilon;
            else
                den = (1.0 - cfg->alpha) * local + cfg->alpha * max_pupil + cfg->epsilon;
            s->exit_spec[i] = c_divr(c_mul(c_conj(pup), s->difference[i]), den);
        }
        st = insert_adjoint_c(s->object, s->mh, s->mw, (long)p->start_row[frame], (long)p->start_col[frame], s->h,
                              s->w, src_off_row(p, frame), src_off_col(p, frame), s->exit_spec,
                              fw * cfg->object_step * normalized);
        if (st) return st;
        if (cfg->has_pupil_step) {
            double max_object = 0.0;
            for (size_t i = 0; i < n; ++i) max_object = fmax(max_object, c_norm_sqr(s->patch[i]));
            max_object = fmax(max_object, cfg->epsilon);
            for (size_t i = 0; i < n; ++i)
                s->pupil_gradient[i] = c_add(s->pupil_gradient[i],
                                             c_divr(c_scale(c_mul(c_conj(s->patch[i]), s->difference[i]), normalized),
                                                    max_object + cfg->epsilon));
            for (size_t i = 0; i < n; ++i)
                s->pupil[i] = c_add(s->pupil[i], c_scale(s->pupil_gradient[i], fw * cfg->pupil_step));
            if (cfg->constrain_pupil)
                for (size_t i = 0; i < n; ++i)
                    if (p->support[i] == 0) s->pupil[i] = cx(0.0, 0.0);
        }
        if (cfg->momentum) {
            s->momentum_count += 1;
            if (s->momentum_count >= cfg->interval) {
                if (s->momentum_count != cfg->interval)
                    return fail(ORC_INVALID_MODEL, "mPIE frame counter exceeds the configured momentum interval");
                st = orc_momentum_event((double *)s->object, (double *)s->velocity, (double *)s->anchor,
                                        (int64_t)s->n_high, cfg->friction, cfg->feedback);
                if (st) return st;
                s->momentum_count = 0;
            }
        }
    }
    return ORC_OK;
}

/* GradientDescent::step (src/algorithms/gradient_descent.rs:405-671) for the
 * ordinary object gradient: no truncation, pupil or illumination recovery,
 * and no regularisation. */
/* truncation_accepts (src/algorithms/gradient_descent.rs:1180-1182). */
int32_t orc_truncation_accepts(double predicted, double measured, double scale) {
    return fabs(measured - predicted) <= scale * sqrt(fmax(predicted, 0.0));
}

/* compute_truncation_statistics (src/algorithms/gradient_descent.rs:701-792):
 * frame-weighted mean absolute residual of the batch's unmasked pixels over
 * the object RMS amplitude, times the threshold. */
static int32_t truncation_scale(orc_state *s, const int *frames, int count, double threshold, double epsilon,
                                double *scale) {
    const orc_problem *p = s->p;
    size_t n = s->n_low;
    double residual_sum = 0.0, pixel_weight = 0.0;
    for (int b = 0; b < count; ++b) {
        int frame = frames[b];
        double fw = frame_weight(p, frame);
        if (fw == 0.0) continue;
        int32_t st = source_field(s, frame);
        if (st) return st;
        const double *measured = p->data + (size_t)frame * n;
        const uint8_t *mask = frame_mask(p, frame);
        double gain = s->gains[frame];
        if (!isfinite(gain) || gain <= 0.0) return fail(ORC_INVALID_MODEL, "state frame %d has invalid gain", frame);
        long valid = 0;
        for (size_t i = 0; i < n; ++i) {
            if (mask && mask[i] == 0) continue;
            ++valid;
            double predicted = fmax(c_norm_sqr(s->field[i]), 0.0);
            double target = fmax((measured[i] - state_background(s, frame, i)) / gain, 0.0);
            residual_sum += fw * fabs(target - predicted);
            pixel_weight += fw;
        }
        if (valid == 0) return fail(ORC_INVALID_MEASUREMENTS, "frame %d has no unmasked pixels", frame);
    }
    double norm = 0.0;
    for (size_t i = 0; i < s->n_high; ++i) norm += c_norm_sqr(s->object[i]);
    double object_rms = fmax(sqrt(norm), sqrt(epsilon));
    double mean_residual = pixel_weight > 0.0 ? residual_sum / pixel_weight : 0.0;
    *scale = threshold * mean_residual / object_rms;
    if (!isfinite(*scale) || *scale < 0.0) return fail(ORC_NUMERICAL, "Poisson truncation statistic is non-finite");
    return ORC_OK;
}

/* Pupil recovery of GradientDescent::step (src/algorithms/gradient_descent.rs:
 * 563-577, 624-640, 654-656): per frame the pupil gradient adds
 * w * (N^2 / valid) * conj(patch) * spectrum / (max |patch|^2 + eps); at
 * the batch end the pupil moves by pupil_step / active frames, then the
 * support is imposed. */
typedef struct {
    int recover;
    double step;
    int constrain;
    double tv_weight, tv_epsilon;  /* object TV regulariser (0: off) */
    double smoothing;              /* pupil quadratic smoothing (0: off) */
    int illumination;              /* finite-difference source-offset recovery */
    double illumination_step, illumination_distance, illumination_bounds;
} gd_pupil_config;

/* CropIndices::validate_subpixel_inside (src/model/crop.rs:105-113). */
static int offset_valid(const orc_problem *p, int source, double orow, double ocol) {
    axis_interp a;
    return interpolation_axis((long)p->start_row[source], p->h, p->mh, orow, &a) == ORC_OK &&
           interpolation_axis((long)p->start_col[source], p->w, p->mw, ocol, &a) == ORC_OK;
}

/* |field|^2 of one source at the given offsets (compute_source_field,
 * src/algorithms/gradient_descent.rs:1184-1213). */
static int32_t intensity_at(orc_state *s, int source, double orow, double ocol, double *out) {
    const orc_problem *p = s->p;
    int32_t st = extract_patch_c(s->object, s->mh, s->mw, (long)p->start_row[source], (long)p->start_col[source],
                                 s->h, s->w, orow, ocol, s->fd_patch);
    if (st) return st;
    for (size_t i = 0; i < s->n_low; ++i) s->fd_patch[i] = c_mul(s->fd_patch[i], s->pupil[i]);
    ifftshift_c(s->fd_patch, s->fd_field, s->h, s->w);
    fft2_c(s->fd_field, s->h, s->w, 1);
    for (size_t i = 0; i < s->n_low; ++i) out[i] = c_norm_sqr(s->fd_field[i]);
    return ORC_OK;
}

/* descent_curvature (src/algorithms/gradient_descent.rs:1340-1360). */
static double descent_curvature(double predicted, double factor, int loss, double epsilon) {
    double mean = fmax(predicted, epsilon);
    switch (loss) {
    case ORC_LOSS_AMPLITUDE_MSE: return 0.5 / mean;
    case ORC_LOSS_INTENSITY_MSE: return 2.0;
    case ORC_LOSS_POISSON_NLL: return 1.0 / mean;
    default: {
        double clipped = factor * 2.0 * sqrt(mean);
        return fabs(clipped) < 1.0 ? 0.25 / mean : epsilon;
    }
    }
}

/* illumination_axis_gradient (src/algorithms/gradient_descent.rs:1272-1338):
 * central (or one-sided at the grid edge) differences of the frame's
 * intensity along one offset axis, chained with the loss derivative and its
 * Gauss-Newton curvature over the retained pixels. */
static int32_t illumination_axis(orc_state *s, int source, double orow, double ocol, double drow, double dcol, int loss,
                                 double epsilon, double *gradient, double *curvature) {
    double distance = fabs(drow) + fabs(dcol);
    int plus_valid = offset_valid(s->p, source, orow + drow, ocol + dcol);
    int minus_valid = offset_valid(s->p, source, orow - drow, ocol - dcol);
    *gradient = *curvature = 0.0;
    if (!plus_valid && !minus_valid) return ORC_OK;
    int32_t st = ORC_OK;
    if (plus_valid) st = intensity_at(s, source, orow + drow, ocol + dcol, s->fd_plus);
    if (!st && minus_valid) st = intensity_at(s, source, orow - drow, ocol - dcol, s->fd_minus);
    if (st) return st;
    for (size_t i = 0; i < s->n_low; ++i) {
        if (!s->dgmask[i]) continue;
        double derivative = plus_valid && minus_valid ? (s->fd_plus[i] - s->fd_minus[i]) / (2.0 * distance)
                            : plus_valid            ? (s->fd_plus[i] - s->calref[i]) / distance
                                                    : (s->calref[i] - s->fd_minus[i]) / distance;
        double factor = s->projected[i].re, predicted = s->projected[i].im;
        *gradient += factor * derivative;
        *curvature += descent_curvature(predicted, factor, loss, epsilon) * derivative * derivative;
    }
    return ORC_OK;
}

/* apply_illumination_update (src/algorithms/gradient_descent.rs:1044-1089):
 * a bounded Gauss-Newton step on each source's correction, kept only when
 * the corrected crop stays inside the grid. */
static int32_t illumination_update(orc_state *s, const gd_pupil_config *cfg, double epsilon) {
    for (int src = 0; src < s->frames; ++src) {
        const double *acc = s->ill + 5 * (size_t)src;
        if (acc[4] == 0.0) continue;
        if (!isfinite(acc[0]) || !isfinite(acc[1]) || !isfinite(acc[2]) || !isfinite(acc[3]) || acc[2] < 0.0 ||
            acc[3] < 0.0)
            return fail(ORC_NUMERICAL, "illumination gradient or curvature for source %d is invalid", src);
        double b = cfg->illumination_bounds;
        double cr = fmin(fmax(s->corr[2 * src] - cfg->illumination_step * acc[0] / (acc[2] + epsilon), -b), b);
        double cc = fmin(fmax(s->corr[2 * src + 1] - cfg->illumination_step * acc[1] / (acc[3] + epsilon), -b), b);
        if (offset_valid(s->p, src, src_off_row(s->p, src) + cr, src_off_col(s->p, src) + cc)) {
            s->corr[2 * src] = cr;
            s->corr[2 * src + 1] = cc;
        }
    }
    return ORC_OK;
}

/* apply_complex_tv_step (src/algorithms/regularization.rs:5-48): one step of
 * the smoothed isotropic TV gradient, accumulated in the reference's order. */
static int32_t complex_tv_step(cplx *values, int h, int w, double weight, double epsilon) {
    if (weight == 0.0 || h <= 0 || w <= 0) return ORC_OK;
    size_t n = (size_t)h * w;
    cplx *gradient = (cplx *)calloc(n, sizeof(cplx));
    for (int row = 0; row < h; ++row)
        for (int col = 0; col < w; ++col) {
            size_t px = (size_t)row * w + col;
            int has_h = col + 1 < w, has_v = row + 1 < h;
            cplx dh = has_h ? c_sub(values[px + 1], values[px]) : cx(0.0, 0.0);
            cplx dv = has_v ? c_sub(values[px + w], values[px]) : cx(0.0, 0.0);
            double norm = sqrt((has_h ? c_norm_sqr(dh) : 0.0) + (has_v ? c_norm_sqr(dv) : 0.0) + epsilon * epsilon);
            if (has_h) {
                cplx q = c_divr(dh, norm);
                gradient[px] = c_sub(gradient[px], q);
                gradient[px + 1] = c_add(gradient[px + 1], q);
            }
            if (has_v) {
                cplx q = c_divr(dv, norm);
                gradient[px] = c_sub(gradient[px], q);
                gradient[px + w] = c_add(gradient[px + w], q);
            }
        }
    int32_t st = ORC_OK;
    for (size_t i = 0; i < n; ++i) {
        values[i] = c_sub(values[i], c_scale(gradient[i], weight));
        if (!isfinite(values[i].re) || !isfinite(values[i].im)) st = ORC_NUMERICAL;
    }
    free(gradient);
    return st ? fail(ORC_NUMERICAL, "regularization produced a non-finite value") : ORC_OK;
}

/* apply_quadratic_smoothing_step (src/algorithms/regularization.rs:50-80). */
static int32_t quadratic_smoothing_step(cplx *values, int h, int w, double weight) {
    if (weight == 0.0 || h <= 0 || w <= 0) return ORC_OK;
    size_t n = (size_t)h * w;
    cplx *gradient = (cplx *)calloc(n, sizeof(cplx));
    for (int row = 0; row < h; ++row)
        for (int col = 0; col < w; ++col) {
            size_t px = (size_t)row * w + col;
            if (col + 1 < w) {
                cplx d = c_sub(values[px + 1], values[px]);
                gradient[px] = c_sub(gradient[px], c_scale(d, 2.0));
                gradient[px + 1] = c_add(gradient[px + 1], c_scale(d, 2.0));
            }
            if (row + 1 < h) {
                cplx d = c_sub(values[px + w], values[px]);
                gradient[px] = c_sub(gradient[px], c_scale(d, 2.0));
                gradient[px + w] = c_add(gradient[px + w], c_scale(d, 2.0));
            }
        }
    int32_t st = ORC_OK;
    for (size_t i = 0; i < n; ++i) {
        values[i] = c_sub(values[i], c_scale(gradient[i], weight));
        if (!isfinite(values[i].re) || !isfinite(values[i].im)) st = ORC_NUMERICAL;
    }
    free(gradient);
    return st ? fail(ORC_NUMERICAL, "regularization produced a non-finite value") : ORC_OK;
}

/* apply_object_tv (src/algorithms/gradient_descent.rs:1125-1165): the TV
 * step on the real-space object, through ifftshift, inverse FFT, forward FFT
 * and fftshift of the centred spectrum. */
static int32_t object_tv(orc_state *s, double weight, double epsilon) {
    cplx *field = (cplx *)malloc(sizeof(cplx) * s->n_high);
    ifftshift_c(s->object, field, s->mh, s->mw);
    fft2_c(field, s->mh, s->mw, 1);
    int32_t st = complex_tv_step(field, s->mh, s->mw, weight, epsilon);
    if (!st) {
        fft2_c(field, s->mh, s->mw, 0);
        fftshift_c(field, s->object, s->mh, s->mw);
    }
    free(field);
    return st;
}

static int32_t gradient_step(orc_state *s, const int *frames, int count, double object_step, double epsilon,
                             int loss, double truncation_threshold, const gd_pupil_config *pupil_cfg,
                             step_summary *summary) {
    const orc_problem *p = s->p;
    size_t n = s->n_low;
    double scale = 0.0;
    const int truncate = truncation_threshold > 0.0;
    if (truncate) {
        int32_t st = truncation_scale(s, frames, count, truncation_threshold, epsilon, &scale);
        if (st) return st;
    }
    double max_pupil = 0.0;
    for (size_t i = 0; i < n; ++i) max_pupil = fmax(max_pupil, c_norm_sqr(s->pupil[i]));
    max_pupil = fmax(max_pupil, epsilon);
    if (!s->gradient) s->gradient = (cplx *)malloc(sizeof(cplx) * s->n_high);
    memset(s->gradient, 0, sizeof(cplx) * s->n_high);
    const int recover_pupil = pupil_cfg && pupil_cfg->recover;
    if (recover_pupil) memset(s->pupil_gradient, 0, sizeof(cplx) * n);
    const int illumination = pupil_cfg && pupil_cfg->illumination && s->corr;
    if (illumination) memset(s->ill, 0, sizeof(double) * 5 * (size_t)s->frames);
    long active = 0;
    for (int b = 0; b < count; ++b) {
        int frame = frames[b];
        double fw = frame_weight(p, frame);
        if (fw == 0.0) continue;
        ++active;
        int32_t st = source_field(s, frame);
        if (st) return st;
        for (size_t i = 0; i < n; ++i) s->projected[i] = cx(c_norm_sqr(s->field[i]), 0.0);
        const double *measured = p->data + (size_t)frame * n;
        const uint8_t *mask = frame_mask(p, frame);
        double gain = s->gains[frame];
        if (!isfinite(gain) || gain <= 0.0) return fail(ORC_INVALID_MODEL, "state frame %d has invalid gain", frame);
        double frame_loss = 0.0;
        long valid = 0;
        for (size_t i = 0; i < n; ++i) {
            if (mask && mask[i] == 0) {
                s->projected[i] = cx(0.0, 0.0);
                if (illumination) s->dgmask[i] = 0;
                continue;
            }
            ++valid;
            double bg = state_background(s, frame, i);
            double intrinsic = fmax(s->projected[i].re, 0.0);
            double target = fmax((measured[i] - bg) / gain, 0.0);
            frame_loss += point_loss(intrinsic, target, loss);
            const int retained = !truncate || orc_truncation_accepts(intrinsic, target, scale);
            if (illumination) s->dgmask[i] = (uint8_t)retained;
            s->projected[i] = cx(retained ? descent_factor(intrinsic, target, loss, epsilon) : 0.0, intrinsic);
        }
        if (valid == 0) return fail(ORC_INVALID_MEASUREMENTS, "frame %d has no unmasked pixels", frame);
        double valid_scale = (double)n / (double)valid;
        summary->objective_sum += fw * (frame_loss / (double)valid);
        summary->weight_sum += fw;
        /* The reference recomputes the same field here; the object has not
         * changed, so the field from above is reused. */
        if (illumination)
            for (size_t i = 0; i < n; ++i) s->calref[i] = c_norm_sqr(s->field[i]);
        for (size_t i = 0; i < n; ++i) s->field[i] = c_scale(s->field[i], 1.0 * s->projected[i].re);
        fft2_c(s->field, s->h, s->w, 0);
        fftshift_c(s->field, s->spectrum, s->h, s->w);
        if (recover_pupil) {
            double max_object = 0.0;
            for (size_t i = 0; i < n; ++i) max_object = fmax(max_object, c_norm_sqr(s->patch[i]));
            max_object = fmax(max_object, epsilon);
            for (size_t i = 0; i < n; ++i)
                s->pupil_gradient[i] = c_add(s->pupil_gradient[i],
                                             c_scale(c_mul(c_conj(s->patch[i]), s->spectrum[i]),
                                                     fw * valid_scale / (max_object + epsilon)));
        }
        for (size_t i = 0; i < n; ++i)
            s->difference[i] = c_divr(c_mul(c_conj(s->pupil[i]), s->spectrum[i]), max_pupil + epsilon);
        st = insert_adjoint_c(s->gradient, s->mh, s->mw, (long)p->start_row[frame], (long)p->start_col[frame], s->h,
                              s->w, eff_off_row(s, frame), eff_off_col(s, frame), s->difference, fw * valid_scale);
        if (st) return st;
        if (illumination) {
            /* illumination_gradient (src/algorithms/gradient_descent.rs:1236-1270). */
            double orow = eff_off_row(s, frame), ocol = eff_off_col(s, frame), d = pupil_cfg->illumination_distance;
            double gr, cr, gc, cc;
            st = illumination_axis(s, frame, orow, ocol, d, 0.0, loss, epsilon, &gr, &cr);
            if (!st) st = illumination_axis(s, frame, orow, ocol, 0.0, d, loss, epsilon, &gc, &cc);
            if (st) return st;
            double *acc = s->ill + 5 * (size_t)frame;
            acc[0] += fw * (gr / (double)valid);
            acc[1] += fw * (gc / (double)valid);
            acc[2] += fw * (cr / (double)valid);
            acc[3] += fw * (cc / (double)valid);
            acc[4] += fw;
        }
    }
    if (active > 0) {
        double step = object_step / (double)active;
        for (size_t i = 0; i < s->n_high; ++i) s->object[i] = c_sub(s->object[i], c_scale(s->gradient[i], step));
        if (recover_pupil) {
            double pstep = pupil_cfg->step / (double)active;
            for (size_t i = 0; i < n; ++i) {
                s->pupil[i] = c_sub(s->pupil[i], c_scale(s->pupil_gradient[i], pstep));
                if (!isfinite(s->pupil[i].re) || !isfinite(s->pupil[i].im))
                    return fail(ORC_NUMERICAL, "pupil update produced a non-finite value");
            }
        }
    }
    /* Regularisers at the batch end, scaled by the batch's share of the
     * frames (src/algorithms/gradient_descent.rs:643-660). */
    double batch_fraction = (double)count / (double)s->frames;
    if (pupil_cfg && pupil_cfg->tv_weight > 0.0) {
        int32_t st = object_tv(s, batch_fraction * pupil_cfg->tv_weight, pupil_cfg->tv_epsilon);
        if (st) return st;
    }
    if (recover_pupil && pupil_cfg->smoothing > 0.0) {
        int32_t st = quadratic_smoothing_step(s->pupil, s->h, s->w, batch_fraction * pupil_cfg->smoothing);
        if (st) return st;
    }
    if (recover_pupil && pupil_cfg->constrain) {
        const uint8_t *support = s->p->support;
        for (size_t i = 0; i < n; ++i)
            if (support[i] == 0) s->pupil[i] = cx(0.0, 0.0);
    }
    if (illumination) return illumination_update(s, pupil_cfg, epsilon);
    return ORC_OK;
}

/* ---------------------------------------------------------------- gauge */

/* relative_phase_slope (src/algorithms/gauge.rs:75-130). */
static double relative_phase_slope(const orc_state *s, int axis_row, double tol) {
    const cplx *values = s->pupil, *ref = (const cplx *)s->p->pupil;
    const uint8_t *support = s->p->support;
    int h = s->h, w = s->w;
    cplx resultant = cx(0, 0), strongest = cx(0, 0);
    double total = 0.0, strongest_w = 0.0;
    int rl = axis_row ? h - 1 : h, cl = axis_row ? w : w - 1;
    for (int r = 0; r < rl; ++r)
        for (int c = 0; c < cl; ++c) {
            size_t cur = (size_t)r * w + c;
            size_t nxt = axis_row ? (size_t)(r + 1) * w + c : cur + 1;
            if (support[cur] == 0 || support[nxt] == 0) continue;
            cplx ce = c_mul(values[nxt], c_conj(values[cur]));
            cplx re = c_mul(ref[nxt], c_conj(ref[cur]));
            cplx contribution = c_mul(ce, c_conj(re));
            double weight = c_norm(contribution);
            if (!isfinite(weight)) continue;
            resultant = c_add(resultant, contribution);
            total += weight;
            if (weight > strongest_w) {
                strongest = contribution;
                strongest_w = weight;
            }
        }
    if (total == 0.0) return 0.0;
    if (c_norm(resultant) > tol * total) return c_arg(resultant);
    if (strongest_w > 0.0) return c_arg(strongest);
    return 0.0;
}

/* canonicalize_object_pupil (src/algorithms/gauge.rs:20-73) with
 * apply_affine_correction (:132-156), normalize_pupil_scale_and_phase
 * (:158-240) and normalize_object_phase (:242-282). */
static int32_t canonicalize_gauge(orc_state *s) {
    const orc_problem *p = s->p;
    size_t n = s->n_low;
    long support_count = 0;
    for (size_t i = 0; i < n; ++i) support_count += p->support[i] != 0;
    if (support_count == 0) return fail(ORC_INVALID_MODEL, "compiled reference pupil support is empty");
    double tol = 64.0 * 2.220446049250313e-16 * (double)support_count;
    int row_exact = 1, col_exact = 1;
    /* The effective offsets, recovered illumination corrections included (gauge.rs:48-52). */
    for (int src = 0; src < s->frames; ++src) {
        row_exact &= offset_is_zero(eff_off_row(s, src), 0.0);
        col_exact &= offset_is_zero(0.0, eff_off_col(s, src));
    }
    double row_slope = row_exact ? relative_phase_slope(s, 1, tol) : 0.0;
    double col_slope = col_exact ? relative_phase_slope(s, 0, tol) : 0.0;
    if (fabs(row_slope) > tol || fabs(col_slope) > tol) {
        for (int r = 0; r < s->h; ++r) {
            double y = (double)r - (double)(s->h / 2);
            for (int c = 0; c < s->w; ++c) {
                double x = (double)c - (double)(s->w / 2);
                s->pupil[(size_t)r * s->w + c] =
                    c_mul(s->pupil[(size_t)r * s->w + c], c_polar(1.0, -(row_slope * y + col_slope * x)));
            }
        }
        for (int r = 0; r < s->mh; ++r) {
            double y = (double)r - (double)(s->mh / 2);
            for (int c = 0; c < s->mw; ++c) {
                double x = (double)c - (double)(s->mw / 2);
                s->object[(size_t)r * s->mw + c] =
                    c_mul(s->object[(size_t)r * s->mw + c], c_polar(1.0, row_slope * y + col_slope * x));
            }
        }
    }
    const cplx *ref = (const cplx *)p->pupil;
    double ref_energy = 0.0, cur_energy = 0.0;
    for (size_t i = 0; i < n; ++i)
        if (p->support[i]) {
            ref_energy += c_norm_sqr(ref[i]);
            cur_energy += c_norm_sqr(s->pupil[i]);
        }
    if (!isfinite(ref_energy) || ref_energy <= 0.0)
        return fail(ORC_INVALID_MODEL, "compiled reference pupil has invalid supported energy");
    if (!isfinite(cur_energy) || cur_energy <= 0.0)
        return fail(ORC_NUMERICAL, "object/pupil gauge normalization requires positive finite recovered pupil energy");
    double computed = sqrt(ref_energy / cur_energy);
    if (!isfinite(computed) || computed <= 0.0)
        return fail(ORC_NUMERICAL, "object/pupil gauge normalization produced an invalid pupil scale");
    double scale = fabs(computed - 1.0) <= tol ? 1.0 : computed;
    cplx overlap = cx(0, 0), strongest = cx(0, 0);
    double overlap_w = 0.0, strongest_w = 0.0;
    for (size_t i = 0; i < n; ++i) {
        if (p->support[i] == 0) continue;
        cplx contribution = c_mul(c_conj(ref[i]), s->pupil[i]);
        double weight = c_norm(contribution);
        overlap = c_add(overlap, contribution);
        overlap_w += weight;
        if (weight > strongest_w) {
            strongest = contribution;
            strongest_w = weight;
        }
    }
    double phase;
    if (overlap_w > 0.0 && c_norm(overlap) > tol * overlap_w)
        phase = c_arg(overlap);
    else if (strongest_w > 0.0)
        phase = c_arg(strongest);
    else
        return fail(ORC_NUMERICAL, "object/pupil gauge normalization could not anchor recovered pupil phase");
    if (!isfinite(phase)) return fail(ORC_NUMERICAL, "object/pupil gauge normalization produced a non-finite pupil phase");
    if (fabs(phase) <= tol) phase = 0.0;
    cplx pupil_factor = c_polar(scale, -phase);
    cplx object_factor = c_div(cx(1.0, 0.0), pupil_factor);
    if (!(pupil_factor.re == 1.0 && pupil_factor.im == 0.0)) {
        for (size_t i = 0; i < n; ++i) s->pupil[i] = c_mul(s->pupil[i], pupil_factor);
        for (size_t i = 0; i < s->n_high; ++i) s->object[i] = c_mul(s->object[i], object_factor);
    }
    cplx strongest_o = cx(0, 0);
    double strongest_m = 0.0;
    for (size_t i = 0; i < s->n_high; ++i) {
        cplx v = s->object[i];
        if (!isfinite(v.re) || !isfinite(v.im))
            return fail(ORC_NUMERICAL, "object/pupil gauge normalization requires a finite object spectrum");
        double m = c_norm(v);
        if (m > strongest_m) {
            strongest_o = v;
            strongest_m = m;
        }
    }
    if (strongest_m == 0.0) return ORC_OK;
    cplx dc = s->object[(size_t)(s->mh / 2) * s->mw + s->mw / 2];
    cplx anchor = c_norm(dc) > tol * strongest_m ? dc : strongest_o;
    double object_phase = c_arg(anchor);
    if (!isfinite(object_phase)) return fail(ORC_NUMERICAL, "object/pupil gauge normalization produced a non-finite object phase");
    if (fabs(object_phase) <= tol) return ORC_OK;
    cplx correction = c_polar(1.0, -object_phase);
    for (size_t i = 0; i < s->n_high; ++i) s->object[i] = c_mul(s->object[i], correction);
    return ORC_OK;
}

/* ------------------------------------------------------------- schedule */

/* f64::total_cmp ordering key. */
static int64_t total_key(double v) {
    int64_t bits;
    memcpy(&bits, &v, sizeof bits);
    bits ^= (int64_t)(((uint64_t)(bits >> 63)) >> 1);
    return bits;
}

typedef struct {
    int frame;
    double a, b;
} sort_item;

static int cmp_items(const void *x, const void *y) {
    const sort_item *l = (const sort_item *)x, *r = (const sort_item *)y;
    int64_t la = total_key(l->a), ra = total_key(r->a);
    if (la != ra) return la < ra ? -1 : 1;
    int64_t lb = total_key(l->b), rb = total_key(r->b);
    if (lb != rb) return lb < rb ? -1 : 1;
    return l->frame < r->frame ? -1 : (l->frame > r->frame);
}

/* FrameSchedule::order / order_for_problem (src/reconstruction/schedule.rs:35-102). */
static int32_t schedule_order(const orc_problem *p, int schedule, int *order) {
    int frames = p->frames;
    for (int f = 0; f < frames; ++f) order[f] = f;
    if (schedule == ORC_SCHEDULE_SEQUENTIAL) return ORC_OK;
    sort_item *items = (sort_item *)malloc(sizeof(sort_item) * (size_t)frames);
    for (int f = 0; f < frames; ++f) {
        items[f].frame = f;
        items[f].b = 0.0;
        if (schedule == ORC_SCHEDULE_SNR_WEIGHTED) {
            double w = frame_weight(p, f);
            double score;
            if (w == 0.0) {
                score = -INFINITY;
            } else {
                size_t n = (size_t)p->h * p->w;
                const double *m = p->data + (size_t)f * n;
                const uint8_t *mask = frame_mask(p, f);
                double sum = 0.0;
                long valid = 0;
                for (size_t i = 0; i < n; ++i)
                    if (!mask || mask[i] != 0) {
                        sum += fmax(m[i] - model_background(p, f, i), 0.0);
                        ++valid;
                    }
                score = valid == 0 ? -INFINITY : w * sqrt(sum / (double)valid);
            }
            items[f].a = -score; /* descending score, then ascending frame */
        } else {
            double kx = p->kx[f], ky = p->ky[f];
            items[f].a = hypot(kx, ky);
            if (schedule == ORC_SCHEDULE_SPIRAL_OUT) {
                double angle = fmod(atan2(ky, kx), 2.0 * M_PI);
                if (angle < 0.0) angle += 2.0 * M_PI;
                items[f].b = angle;
            }
        }
    }
    qsort(items, (size_t)frames, sizeof(sort_item), cmp_items);
    for (int f = 0; f < frames; ++f) order[f] = items[f].frame;
    free(items);
    return ORC_OK;
}

/* --------------------------------------------------------------- runner */

/* Runner::run (src/reconstruction/runner.rs:76-285) without callbacks,
 * checkpoints or diagnostics, then ReconstructionResult::from_state
 * (src/reconstruction/result.rs:76-105,397-413). */
int32_t orc_run(const orc_problem *p, const orc_params *prm, orc_output *out) {
    if (prm->batch_size <= 0) return out->status = fail(ORC_INVALID_PARAMETER, "batch_size must be greater than zero");
    if (!isfinite(prm->object_step) || prm->object_step <= 0.0)
        return out->status = fail(ORC_INVALID_PARAMETER, "object_step must be finite and positive");
    if (!isfinite(prm->epsilon) || prm->epsilon <= 0.0)
        return out->status = fail(ORC_INVALID_PARAMETER, "epsilon must be finite and positive");
    if (prm->algorithm == ORC_ALG_GD && prm->recover_pupil && (!isfinite(prm->pupil_step) || prm->pupil_step <= 0.0))
        return out->status = fail(ORC_INVALID_PARAMETER, "pupil_step must be finite and positive");
    /* AdaptiveAlternatingProjection::validate (src/algorithms/adaptive_alternating_projection.rs:350-403). */
    if (prm->algorithm == ORC_ALG_ADAPTIVE_AP) {
        if (prm->iterations == 0) return out->status = fail(ORC_INVALID_PARAMETER, "iterations must be greater than zero");
        if (!isfinite(prm->progress_threshold) || prm->progress_threshold < 0.0 || prm->progress_threshold >= 1.0)
            return out->status = fail(ORC_INVALID_PARAMETER, "progress_threshold must be in [0, 1)");
        if (!isfinite(prm->reduction_factor) || prm->reduction_factor <= 0.0 || prm->reduction_factor >= 1.0)
            return out->status = fail(ORC_INVALID_PARAMETER, "reduction_factor must be in (0, 1)");
        if (!isfinite(prm->minimum_object_step) || prm->minimum_object_step <= 0.0 ||
            prm->minimum_object_step > prm->object_step)
            return out->status = fail(ORC_INVALID_PARAMETER, "minimum_object_step must be positive and at most the initial step");
    }
    /* GradientDescent::validate (src/algorithms/gradient_descent.rs:319-331). */
    if (prm->poisson_truncation_threshold != 0.0) {
        if (!isfinite(prm->poisson_truncation_threshold) || prm->poisson_truncation_threshold < 0.0)
            return out->status = fail(ORC_INVALID_PARAMETER, "poisson_truncation_threshold must be finite and positive");
        if (prm->loss_type != ORC_LOSS_POISSON_NLL)
            return out->status = fail(ORC_INVALID_PARAMETER, "poisson_truncation_threshold requires Poisson negative log likelihood");
    }
    orc_state s;
    int32_t st = state_init(&s, p);
    if (st) {
        state_free(&s);
        return out->status = st;
    }
    /* A given start state replaces the measured-amplitude initialisation
     * (ReconstructionState::from_object, src/reconstruction/state.rs:357-383). */
    if (prm->initial_spectrum) memcpy(s.object, prm->initial_spectrum, sizeof(cplx) * s.n_high);
    update_config cfg;
    memset(&cfg, 0, sizeof cfg);
    cfg.object_step = prm->object_step;
    cfg.epsilon = prm->epsilon;
    cfg.loss = prm->loss_type;
    cfg.constrain_pupil = 1;
    int canonical = 0;
    switch (prm->algorithm) {
    case ORC_ALG_AP:
    case ORC_ALG_ADAPTIVE_AP:
        cfg.denominator = 0;
        break;
    case ORC_ALG_FPIE:
        cfg.denominator = 1;
        cfg.alpha = prm->stability;
        break;
    case ORC_ALG_MPIE:
        cfg.denominator = 1;
        cfg.alpha = prm->stability;
        cfg.momentum = 1;
        cfg.interval = prm->momentum_interval;
        cfg.friction = prm->momentum_friction;
        cfg.feedback = prm->momentum_feedback;
        s.velocity = (cplx *)calloc(s.n_high, sizeof(cplx));
        s.anchor = (cplx *)malloc(sizeof(cplx) * s.n_high);
        memcpy(s.anchor, s.object, sizeof(cplx) * s.n_high);
        break;
    case ORC_ALG_EPRY:
        cfg.denominator = 2;
        cfg.has_pupil_step = prm->recover_pupil;
        cfg.pupil_step = prm->pupil_step;
        cfg.constrain_pupil = prm->constrain_pupil;
        cfg.gain_update = prm->recover_gains;
        cfg.gain_step = prm->gain_step;
        cfg.gain_min = prm->gain_min;
        cfg.gain_max = prm->gain_max;
        cfg.background_update = prm->recover_background;
        cfg.background_step = prm->background_step;
        cfg.background_min = prm->background_min;
        cfg.background_max = prm->background_max;
        canonical = prm->recover_pupil;
        break;
    case ORC_ALG_GD:
        canonical = prm->recover_pupil;
        break;
    default:
        state_free(&s);
        return out->status = fail(ORC_UNSUPPORTED, "unknown algorithm");
    }
    if (canonical && (st = canonicalize_gauge(&s))) {
        state_free(&s);
        return out->status = st;
    }
    /* AdaptiveAlternatingProjection::begin_iteration
     * (src/algorithms/adaptive_alternating_projection.rs:245-307): the step
     * shrinks by reduction_factor (not below the minimum) when a pass's
     * relative objective progress is at most progress_threshold. */
    const int adaptive = prm->algorithm == ORC_ALG_ADAPTIVE_AP;
    double previous_objective = NAN, last_objective = NAN;
    int *order = (int *)malloc(sizeof(int) * (size_t)p->frames);
    for (int it = 0; it < prm->iterations && !st; ++it) {
        if (adaptive && it > 0) {
            if (!isfinite(last_objective) || last_objective < 0.0) {
                st = fail(ORC_NUMERICAL, "adaptive alternating projection produced an invalid pass objective");
                break;
            }
            if (isfinite(previous_objective)) {
                double progress = (previous_objective - last_objective) / fmax(previous_objective, prm->epsilon);
                if (progress <= prm->progress_threshold)
                    cfg.object_step = fmax(cfg.object_step * prm->reduction_factor, prm->minimum_object_step);
            }
            previous_objective = last_objective;
        }
        if (out->object_steps) out->object_steps[it] = cfg.object_step;
        st = schedule_order(p, prm->schedule, order);
        step_summary summary = {0.0, 0.0};
        for (int start = 0; start < p->frames && !st; start += prm->batch_size) {
            int count = p->frames - start < prm->batch_size ? p->frames - start : prm->batch_size;
            if (prm->algorithm == ORC_ALG_GD)
            {
                const gd_pupil_config pc = {prm->recover_pupil, prm->pupil_step, prm->constrain_pupil,
                                            prm->object_tv_weight, prm->object_tv_epsilon,
                                            prm->pupil_smoothing_weight, prm->recover_illumination,
                                            prm->illumination_step, prm->illumination_finite_difference,
                                            prm->illumination_bounds};
                if (prm->recover_illumination && !s.corr) illumination_alloc(&s);
                st = gradient_step(&s, order + start, count, prm->object_step, prm->epsilon, prm->loss_type,
                                   prm->poisson_truncation_threshold, &pc, &summary);
            }
            else
                st = projection_update(&s, order + start, count, &cfg, &summary);
        }
        if (!st && canonical) st = canonicalize_gauge(&s);
        last_objective = summary.weight_sum > 0.0 ? summary.objective_sum / summary.weight_sum : NAN;
        if (out->objectives) out->objectives[it] = last_objective;
    }
    free(order);
    if (!st) {
        if (out->object_spectrum) memcpy(out->object_spectrum, s.object, sizeof(cplx) * s.n_high);
        if (out->pupil) memcpy(out->pupil, s.pupil, sizeof(cplx) * s.n_low);
        if (out->object) {
            ifftshift_c(s.object, (cplx *)out->object, s.mh, s.mw);
            fft2_c((cplx *)out->object, s.mh, s.mw, 1);
        }
        if (out->illumination_corrections)
            for (size_t i = 0; i < 2 * (size_t)s.frames; ++i)
                out->illumination_corrections[i] = s.corr ? s.corr[i] : 0.0;
        if (out->frame_gains) memcpy(out->frame_gains, s.gains, sizeof(double) * (size_t)s.frames);
        if (out->background)
            for (size_t i = 0; i < (size_t)s.frames * s.n_low; ++i)
                out->background[i] = s.background ? s.background[i] : 0.0;
    }
    state_free(&s);
    return out->status = st;
}

/* ------------------------------------------------------------ threading */

typedef struct {
    int32_t count;
    const orc_problem *problems;
    const orc_params *params;
    orc_output *outputs;
    int next;
    pthread_mutex_t lock;
} run_pool;

static void *run_worker(void *arg) {
    run_pool *pool = (run_pool *)arg;
    for (;;) {
        pthread_mutex_lock(&pool->lock);
        int i = pool->next++;
        pthread_mutex_unlock(&pool->lock);
        if (i >= pool->count) break;
        orc_run(&pool->problems[i], pool->params, &pool->outputs[i]);
    }
    return NULL;
}

/* Independent tiles run concurrently; each tile keeps its own sequential
 * frame order exactly as a single run would. */
int32_t orc_run_many(int32_t count, const orc_problem *problems, const orc_params *params,
                     orc_output *outputs, int32_t workers) {
    if (workers < 1) workers = 1;
    if (workers > count) workers = count;
    run_pool pool = {count, problems, params, outputs, 0, PTHREAD_MUTEX_INITIALIZER};
    pthread_t *threads = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)workers);
    for (int t = 0; t < workers; ++t) pthread_create(&threads[t], NULL, run_worker, &pool);
    for (int t = 0; t < workers; ++t) pthread_join(threads[t], NULL);
    free(threads);
    for (int i = 0; i < count; ++i)
        if (outputs[i].status) return outputs[i].status;
    return ORC_OK;
}

/* ------------------------------------------------------ forward, result */

int32_t orc_object_spectrum(const double *object, int32_t mh, int32_t mw, double *spectrum) {
    size_t n = (size_t)mh * mw;
    cplx *tmp = (cplx *)malloc(sizeof(cplx) * n);
    memcpy(tmp, object, sizeof(cplx) * n);
    fft2_c(tmp, mh, mw, 0);
    fftshift_c(tmp, (cplx *)spectrum, mh, mw);
    free(tmp);
    return ORC_OK;
}

int32_t orc_state_object(const double *spectrum, int32_t mh, int32_t mw, double *object) {
    ifftshift_c((const cplx *)spectrum, (cplx *)object, mh, mw);
    fft2_c((cplx *)object, mh, mw, 1);
    return ORC_OK;
}

typedef struct {
    const orc_problem *p;
    const cplx *spectrum;
    double *out;
    int first, last;
    int32_t status;
} forward_job;

/* ForwardModel::forward_intensity_standard_into (src/model/forward.rs:245-292)
 * for a contiguous chunk of frames. */
static void *forward_worker(void *arg) {
    forward_job *job = (forward_job *)arg;
    const orc_problem *p = job->p;
    size_t n = (size_t)p->h * p->w;
    cplx *patch = (cplx *)malloc(sizeof(cplx) * n * 2);
    cplx *field = patch + n;
    const cplx *pupil = (const cplx *)p->pupil;
    for (int f = job->first; f < job->last; ++f) {
        int32_t st = extract_patch_c(job->spectrum, p->mh, p->mw, (long)p->start_row[f], (long)p->start_col[f], p->h,
                                     p->w, src_off_row(p, f), src_off_col(p, f), patch);
        if (st) {
            job->status = st;
            break;
        }
        for (size_t i = 0; i < n; ++i) patch[i] = c_mul(patch[i], pupil[i]);
        ifftshift_c(patch, field, p->h, p->w);
        fft2_c(field, p->h, p->w, 1);
        double gain = model_gain(p, f);
        double *dst = job->out + (size_t)f * n;
        for (size_t i = 0; i < n; ++i) dst[i] = gain * c_norm_sqr(field[i]) + model_background(p, f, i);
    }
    free(patch);
    return NULL;
}

/* ForwardModel::forward_intensity_stack_into (src/model/forward.rs:300-372):
 * contiguous frame chunks per worker; results do not depend on the count. */
int32_t orc_forward_stack(const orc_problem *p, const double *spectrum, double *out, int32_t workers) {
    if (workers <= 0) return fail(ORC_INVALID_PARAMETER, "worker_count must be greater than zero");
    if (workers > p->frames) workers = p->frames;
    int per = (p->frames + workers - 1) / workers;
    int jobs = (p->frames + per - 1) / per;
    forward_job *job = (forward_job *)calloc((size_t)jobs, sizeof(forward_job));
    pthread_t *threads = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)jobs);
    for (int j = 0; j < jobs; ++j) {
        job[j].p = p;
        job[j].spectrum = (const cplx *)spectrum;
        job[j].out = out;
        job[j].first = j * per;
        job[j].last = (j + 1) * per < p->frames ? (j + 1) * per : p->frames;
        pthread_create(&threads[j], NULL, forward_worker, &job[j]);
    }
    int32_t st = ORC_OK;
    for (int j = 0; j < jobs; ++j) {
        pthread_join(threads[j], NULL);
        if (job[j].status && !st) st = job[j].status;
    }
    free(job);
    free(threads);
    return st;
}

/* compare_complex_fields_masked complex_nrmse
 * (src/metrics/complex_field/comparison.rs:60-121), unmasked. */
double orc_complex_nrmse(const double *reference_d, const double *candidate_d, int64_t len) {
    const cplx *reference = (const cplx *)reference_d, *candidate = (const cplx *)candidate_d;
    cplx cross = cx(0, 0);
    for (int64_t i = 0; i < len; ++i) cross = c_add(cross, c_mul(candidate[i], c_conj(reference[i])));
    cplx correction = c_polar(1.0, -c_arg(cross));
    double err = 0.0, ref = 0.0;
    for (int64_t i = 0; i < len; ++i) {
        cplx aligned = c_mul(candidate[i], correction);
        err += c_norm_sqr(c_sub(aligned, reference[i]));
        ref += c_norm_sqr(reference[i]);
    }
    double count = (double)len;
    double denominator = sqrt(ref / count);
    if (denominator < 2.220446049250313e-16) denominator = 2.220446049250313e-16;
    return sqrt(err / count) / denominator;
}

/* ------------------------------------------------- narrowband spectral AP */

typedef struct {
    int channel, source;    /* channel kernel and its global source index */
    int object;             /* stored object index */
    double weight;          /* effective mode weight */
    cplx *field, *exit;     /* detector field and pupil-weighted patch, pre-update */
} spectral_mode;

static int spectral_source(const orc_spectral_problem *p, int channel, int local) {
    int offset = 0;
    for (int c = 0; c < channel; ++c) offset += p->channel_sources[c];
    return offset + local;
}

static double spectral_frame_gain(const orc_spectral_problem *p, int channel, int local) {
    return p->frame_gains ? p->frame_gains[spectral_source(p, channel, local)] : 1.0;
}

static int spectral_object_index(const orc_spectral_problem *p, int channel) {
    return p->shared_object ? 0 : channel;
}

static int spectral_object_count(const orc_spectral_problem *p) { return p->shared_object ? 1 : p->channels; }

/* Coherent field and exit of one channel source from a centred spectrum:
 * ForwardModel::forward_source_field_standard_into (src/model/forward.rs:146-169)
 * and the pupil-weighted patch of SpectralReconstructionState::evaluate_frame
 * (src/reconstruction/spectral.rs:330-385). */
static int32_t spectral_source_field(const orc_spectral_problem *p, const cplx *spectrum, int channel, int source,
                                     cplx *exit, cplx *field) {
    size_t n = (size_t)p->h * p->w;
    int32_t st = extract_patch_c(spectrum, p->mh, p->mw, (long)p->start_row[source], (long)p->start_col[source],
                                 p->h, p->w, p->off_row ? p->off_row[source] : 0.0,
                                 p->off_col ? p->off_col[source] : 0.0, exit);
    if (st) return st;
    const cplx *pupil = (const cplx *)p->pupils + (size_t)channel * n;
    for (size_t i = 0; i < n; ++i) exit[i] = c_mul(exit[i], pupil[i]);
    ifftshift_c(exit, field, p->h, p->w);
    fft2_c(field, p->h, p->w, 1);
    return ORC_OK;
}

/* SpectralReconstructionState::initialize (src/reconstruction/spectral.rs:123-199):
 * weighted, mask-aware measured amplitude per stored object, nearest
 * upsampling to the common grid. objects: object_count*mh*mw complex. */
static int32_t spectral_initial_objects(const orc_spectral_problem *p, cplx *objects) {
    size_t n = (size_t)p->h * p->w;
    double *amplitude = (double *)malloc(sizeof(double) * n);
    double *weights = (double *)malloc(sizeof(double) * n);
    int32_t st = ORC_OK;
    for (int o = 0; o < spectral_object_count(p) && !st; ++o) {
        memset(amplitude, 0, sizeof(double) * n);
        memset(weights, 0, sizeof(double) * n);
        double total_amplitude = 0.0, total_weight = 0.0;
        for (int e = 0; e < p->exposures; ++e) {
            int first = p->contribution_offsets[e], last = p->contribution_offsets[e + 1];
            int uses = 0;
            for (int k = first; k < last; ++k)
                if (spectral_object_index(p, p->contribution_channel[k]) == o) uses = 1;
            if (!uses) continue;
            double fw = p->weights ? p->weights[e] : 1.0;
            if (fw == 0.0) continue;
            double gain = 0.0;
            for (int k = first; k < last; ++k)
                gain += p->contribution_weight[k] *
                        spectral_frame_gain(p, p->contribution_channel[k], p->contribution_local[k]);
            gain *= p->exposure_gain[e];
            if (!isfinite(gain) || gain <= 0.0) {
                st = fail(ORC_NUMERICAL, "spectral initialization gain must be finite and positive");
                break;
            }
            const double *measured = p->data + (size_t)e * n;
            const uint8_t *mask = p->masks ? p->masks + (size_t)e * n : NULL;
            for (size_t i = 0; i < n; ++i) {
                if (mask && mask[i] == 0) continue;
                double value = sqrt(fmax((measured[i] - p->exposure_background[e]) / gain, 0.0));
                amplitude[i] += fw * value;
                weights[i] += fw;
                total_amplitude += fw * value;
                total_weight += fw;
            }
        }
        if (st) break;
        double fallback = total_amplitude / total_weight;
        for (size_t i = 0; i < n; ++i) amplitude[i] = weights[i] > 0.0 ? amplitude[i] / weights[i] : fallback;
        cplx *object = objects + (size_t)o * p->mh * p->mw;
        for (long r = 0; r < p->mh; ++r)
            for (long c = 0; c < p->mw; ++c)
                object[r * p->mw + c] = cx(amplitude[(r * p->h / p->mh) * p->w + c * p->w / p->mw], 0.0);
    }
    free(amplitude);
    free(weights);
    return st;
}

/* One exposure of SpectralAlternatingProjection::step
 * (src/algorithms/spectral.rs:182-271): every mode from the pre-frame state,
 * one amplitude ratio from their weighted intensity sum, then each mode's
 * local-denominator correction into its stored object. */
static int32_t spectral_exposure(const orc_spectral_problem *p, const orc_spectral_params *prm, cplx *spectra, int e,
                                 spectral_mode *modes, double *predicted, cplx *projection, cplx *work, cplx *centered,
                                 double *objective_sum, double *weight_sum_out) {
    size_t n = (size_t)p->h * p->w, n_high = (size_t)p->mh * p->mw;
    double fw = p->weights ? p->weights[e] : 1.0;
    if (fw == 0.0) return ORC_OK;
    int first = p->contribution_offsets[e], last = p->contribution_offsets[e + 1];
    int count = last - first;
    int separate = count == 1;
    double effective_gain = p->exposure_gain[e];
    if (separate)
        effective_gain *= p->contribution_weight[first] *
                          spectral_frame_gain(p, p->contribution_channel[first], p->contribution_local[first]);
    memset(predicted, 0, sizeof(double) * n);
    double weight_sum = 0.0;
    for (int k = 0; k < count; ++k) {
        int channel = p->contribution_channel[first + k], local = p->contribution_local[first + k];
        spectral_mode *m = &modes[k];
        m->channel = channel;
        m->source = spectral_source(p, channel, local);
        m->object = spectral_object_index(p, channel);
        m->weight = separate ? 1.0 : p->contribution_weight[first + k] * spectral_frame_gain(p, channel, local);
        int32_t st = spectral_source_field(p, spectra + (size_t)m->object * n_high, channel, m->source, m->exit,
                                           m->field);
        if (st) return st;
        for (size_t i = 0; i < n; ++i) predicted[i] += m->weight * c_norm_sqr(m->field[i]);
        weight_sum += m->weight;
    }
    const double *measured = p->data + (size_t)e * n;
    const uint8_t *mask = p->masks ? p->masks + (size_t)e * n : NULL;
    double background = p->exposure_background[e];
    double loss = 0.0;
    long valid = 0;
    for (size_t i = 0; i < n; ++i) {
        if (mask && mask[i] == 0) {
            projection[i] = cx(1.0, 0.0);
            continue;
        }
        ++valid;
        loss += point_loss(effective_gain * predicted[i] + background, measured[i], prm->loss_type);
        double target = fmax((measured[i] - background) / effective_gain, 0.0);
        projection[i] = predicted[i] > prm->epsilon ? cx(sqrt(target / predicted[i]), 0.0)
                                                    : cx(0.0, sqrt(target / weight_sum));
    }
    if (valid == 0) return fail(ORC_INVALID_MEASUREMENTS, "frame %d has no unmasked pixels", e);
    *objective_sum += fw * (loss / (double)valid);
    *weight_sum_out += fw;
    for (int k = 0; k < count; ++k) {
        spectral_mode *m = &modes[k];
        const cplx *pupil = (const cplx *)p->pupils + (size_t)m->channel * n;
        for (size_t i = 0; i < n; ++i) {
            if (mask && mask[i] == 0)
                work[i] = m->field[i];
            else if (predicted[i] > prm->epsilon)
                work[i] = c_scale(m->field[i], projection[i].re);
            else
                work[i] = cx(projection[i].im, 0.0);
        }
        fft2_c(work, p->h, p->w, 0);
        fftshift_c(work, centered, p->h, p->w);
        for (size_t i = 0; i < n; ++i)
            work[i] = c_divr(c_mul(c_conj(pupil[i]), c_sub(centered[i], m->exit[i])),
                             c_norm_sqr(pupil[i]) + prm->epsilon);
        int32_t st = insert_adjoint_c(spectra + (size_t)m->object * n_high, p->mh, p->mw,
                                      (long)p->start_row[m->source], (long)p->start_col[m->source], p->h, p->w,
                                      p->off_row ? p->off_row[m->source] : 0.0,
                                      p->off_col ? p->off_col[m->source] : 0.0, work,
                                      fw * prm->object_step * (m->weight / weight_sum));
        if (st) return st;
    }
    return ORC_OK;
}

int32_t orc_spectral_run(const orc_spectral_problem *p, const orc_spectral_params *prm, const int32_t *order,
                         const double *initial_objects, const double *initial_spectra,
                         int32_t completed_iterations, double *spectra_out, double *objectives) {
    if (prm->iterations <= 0 || !(prm->object_step > 0.0) || !isfinite(prm->object_step) ||
        !(prm->epsilon > 0.0) || !isfinite(prm->epsilon))
        return fail(ORC_INVALID_PARAMETER, "spectral AP parameters must be positive and finite");
    if (completed_iterations < 0 || completed_iterations > prm->iterations)
        return fail(ORC_INVALID_PARAMETER, "total target cannot precede checkpoint iterations");
    size_t n = (size_t)p->h * p->w, n_high = (size_t)p->mh * p->mw;
    int objects = spectral_object_count(p);
    cplx *spectra = (cplx *)spectra_out;
    int32_t st = ORC_OK;
    if (initial_spectra) {
        memcpy(spectra, initial_spectra, sizeof(cplx) * n_high * objects);
    } else {
        cplx *natural = (cplx *)malloc(sizeof(cplx) * n_high * objects);
        if (initial_objects)
            memcpy(natural, initial_objects, sizeof(cplx) * n_high * objects);
        else
            st = spectral_initial_objects(p, natural);
        for (int o = 0; o < objects && !st; ++o) {
            fft2_c(natural + (size_t)o * n_high, p->mh, p->mw, 0);
            fftshift_c(natural + (size_t)o * n_high, spectra + (size_t)o * n_high, p->mh, p->mw);
        }
        free(natural);
        if (st) return st;
    }
    int max_count = 1;
    for (int e = 0; e < p->exposures; ++e) {
        int count = p->contribution_offsets[e + 1] - p->contribution_offsets[e];
        if (count > max_count) max_count = count;
    }
    spectral_mode *modes = (spectral_mode *)calloc((size_t)max_count, sizeof(spectral_mode));
    cplx *buffers = (cplx *)malloc(sizeof(cplx) * n * (2 * (size_t)max_count + 3));
    for (int k = 0; k < max_count; ++k) {
        modes[k].field = buffers + (size_t)(2 * k) * n;
        modes[k].exit = buffers + (size_t)(2 * k + 1) * n;
    }
    cplx *projection = buffers + (size_t)(2 * max_count) * n;
    cplx *work = projection + n, *centered = work + n;
    double *predicted = (double *)malloc(sizeof(double) * n);
    for (int it = completed_iterations; it < prm->iterations && !st; ++it) {
        double objective_sum = 0.0, weight_sum = 0.0;
        for (int idx = 0; idx < p->exposures && !st; ++idx) {
            int e = order ? order[idx] : idx;
            st = spectral_exposure(p, prm, spectra, e, modes, predicted, projection, work, centered, &objective_sum,
                                   &weight_sum);
        }
        if (st) break;
        if (!(weight_sum > 0.0)) {
            st = fail(ORC_NUMERICAL, "spectral iteration has no positive frame weight");
            break;
        }
        double objective = objective_sum / weight_sum;
        if (!isfinite(objective)) {
            st = fail(ORC_NUMERICAL, "spectral iteration objective is non-finite");
            break;
        }
        if (objectives) objectives[it - completed_iterations] = objective;
    }
    free(predicted);
    free(buffers);
    free(modes);
    return st;
}

int32_t orc_spectral_forward(const orc_spectral_problem *p, const double *spectra_d, double *out) {
    size_t n = (size_t)p->h * p->w, n_high = (size_t)p->mh * p->mw;
    const cplx *spectra = (const cplx *)spectra_d;
    cplx *exit = (cplx *)malloc(sizeof(cplx) * n * 2);
    cplx *field = exit + n;
    int32_t st = ORC_OK;
    for (int e = 0; e < p->exposures && !st; ++e) {
        double *dst = out + (size_t)e * n;
        memset(dst, 0, sizeof(double) * n);
        for (int k = p->contribution_offsets[e]; k < p->contribution_offsets[e + 1] && !st; ++k) {
            int channel = p->contribution_channel[k], local = p->contribution_local[k];
            int source = spectral_source(p, channel, local);
            st = spectral_source_field(p, spectra + (size_t)spectral_object_index(p, channel) * n_high, channel,
                                       source, exit, field);
            double gain = spectral_frame_gain(p, channel, local), weight = p->contribution_weight[k];
            for (size_t i = 0; i < n && !st; ++i) dst[i] += weight * (gain * c_norm_sqr(field[i]));
        }
        for (size_t i = 0; i < n; ++i) dst[i] = p->exposure_gain[e] * dst[i] + p->exposure_background[e];
    }
    free(exit);
    return st;
}

int32_t orc_complex_tv_step(double *values, int32_t h, int32_t w, double weight, double epsilon) {
    return complex_tv_step((cplx *)values, h, w, weight, epsilon);
}

int32_t orc_quadratic_smoothing_step(double *values, int32_t h, int32_t w, double weight) {
    return quadratic_smoothing_step((cplx *)values, h, w, weight);
}

/* One GradientDescent::step (src/algorithms/gradient_descent.rs:405-671)
 * over the batch `frames`, from the given centred spectrum and pupil; the
 * state after the step is copied out. */
int32_t orc_gd_batch_step(const orc_problem *p, const orc_params *prm, const double *spectrum, const double *pupil,
                          const int32_t *frames, int32_t count, double *spectrum_out, double *pupil_out,
                          double *illumination_gradient_out, double *corrections_inout) {
    orc_state s;
    int32_t st = state_init(&s, p);
    if (st) {
        state_free(&s);
        return st;
    }
    for (int32_t k = 0; k < count; ++k)
        if (frames[k] < 0 || frames[k] >= p->frames) {
            state_free(&s);
            return fail(ORC_FRAME_OUT_OF_RANGE, "frame %d is out of range", frames[k]);
        }
    memcpy(s.object, spectrum, sizeof(cplx) * s.n_high);
    memcpy(s.pupil, pupil, sizeof(cplx) * s.n_low);
    const gd_pupil_config pc = {prm->recover_pupil, prm->pupil_step, prm->constrain_pupil, prm->object_tv_weight,
                                prm->object_tv_epsilon, prm->pupil_smoothing_weight, prm->recover_illumination,
                                prm->illumination_step, prm->illumination_finite_difference,
                                prm->illumination_bounds};
    if (prm->recover_illumination) {
        illumination_alloc(&s);
        if (corrections_inout) memcpy(s.corr, corrections_inout, sizeof(double) * 2 * (size_t)s.frames);
    }
    step_summary summary = {0.0, 0.0};
    st = gradient_step(&s, (const int *)frames, count, prm->object_step, prm->epsilon, prm->loss_type, 0.0, &pc,
                       &summary);
    if (!st) {
        memcpy(spectrum_out, s.object, sizeof(cplx) * s.n_high);
        memcpy(pupil_out, s.pupil, sizeof(cplx) * s.n_low);
        if (corrections_inout && s.corr) memcpy(corrections_inout, s.corr, sizeof(double) * 2 * (size_t)s.frames);
        if (illumination_gradient_out)
            for (int src = 0; src < s.frames; ++src) {
                illumination_gradient_out[2 * src] = s.ill ? s.ill[5 * (size_t)src] : 0.0;
                illumination_gradient_out[2 * src + 1] = s.ill ? s.ill[5 * (size_t)src + 1] : 0.0;
            }
    }
    state_free(&s);
    return st;
}

/* The mean point loss of one frame over its unmasked pixels, for the
 * prediction gain * |psi|^2 + background (objective.rs:14-46 on the frame's
 * forward intensity). */
int32_t orc_frame_loss(const orc_problem *p, const double *spectrum, const double *pupil, int32_t frame, int32_t loss,
                       double *out) {
    orc_state s;
    int32_t st = state_init(&s, p);
    if (st) {
        state_free(&s);
        return st;
    }
    memcpy(s.object, spectrum, sizeof(cplx) * s.n_high);
    memcpy(s.pupil, pupil, sizeof(cplx) * s.n_low);
    st = source_field(&s, frame);
    if (!st) {
        const double *measured = p->data + (size_t)frame * s.n_low;
        const uint8_t *mask = frame_mask(p, frame);
        double sum = 0.0;
        long valid = 0;
        for (size_t i = 0; i < s.n_low; ++i) {
            if (mask && mask[i] == 0) continue;
            double predicted = model_gain(p, frame) * c_norm_sqr(s.field[i]) + model_background(p, frame, i);
            sum += point_loss(predicted, measured[i], loss);
            ++valid;
        }
        *out = valid ? sum / (double)valid : NAN;
    }
    state_free(&s);
    return st;
}

/* canonicalize_object_pupil (src/algorithms/gauge.rs:20-73) applied to the
 * given centred spectrum (mh*mw) and pupil (h*w), in place. */
int32_t orc_canonicalize(const orc_problem *p, double *spectrum, double *pupil) {
    orc_state s;
    int32_t st = state_init(&s, p);
    if (st) {
        state_free(&s);
        return st;
    }
    memcpy(s.object, spectrum, sizeof(cplx) * s.n_high);
    memcpy(s.pupil, pupil, sizeof(cplx) * s.n_low);
    st = canonicalize_gauge(&s);
    if (!st) {
        memcpy(spectrum, s.object, sizeof(cplx) * s.n_high);
        memcpy(pupil, s.pupil, sizeof(cplx) * s.n_low);
    }
    state_free(&s);
    return st;
}
