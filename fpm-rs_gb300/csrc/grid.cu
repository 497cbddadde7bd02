// Whole-grid FP64 kernels that run once per reconstruction (initialise and
// finalise) or once per iteration (EPRY gauge):
//  * mixed-radix Stockham line FFTs of any length (reference convention of
//    CpuBackend::fft2, src/backend/cpu.rs:130-175, applied as rows then
//    columns by the caller),
//  * fftshift / ifftshift conversions between the centred FP32 state and
//    natural-order FP64 scratch (src/model/forward.rs:530-569),
//  * object/pupil gauge canonicalisation (src/algorithms/gauge.rs:20-282).
#include <cuda_runtime.h>
#include <math.h>

#include "kernels.h"

namespace fpm {

__device__ __forceinline__ double2 zmul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 zadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 zconj(double2 a) { return make_double2(a.x, -a.y); }
__device__ __forceinline__ double zabs2(double2 a) { return a.x * a.x + a.y * a.y; }

// One block per line. Stage s with radix R maps input index j + r*n/R to
// output (j / Ns) * Ns * R + j % Ns + q * Ns (Stockham autosort), so lines
// come out in natural order without a permutation pass.
__global__ void fft_lines_kernel(double2* const* arrays, int n, long long stride, long long dist,
                                 const double2* __restrict__ roots, const int* __restrict__ factors, int nfactors,
                                 int inverse, double scale) {
    extern __shared__ double2 zsm[];
    double2* a = zsm;
    double2* b = zsm + n;
    double2* base = arrays[blockIdx.y] + (long long)blockIdx.x * dist;
    for (int k = threadIdx.x; k < n; k += blockDim.x) a[k] = base[(long long)k * stride];
    __syncthreads();
    int ns = 1;
    for (int s = 0; s < nfactors; ++s) {
        const int radix = factors[s];
        const int span = ns * radix;
        const int tw_step = n / span;
        const int in_step = n / radix;
        for (int o = threadIdx.x; o < n; o += blockDim.x) {
            const int q = (o / ns) % radix;
            const int j = (o / span) * ns + (o % ns);
            const int e0 = (j % ns) + q * ns;
            double2 sum = make_double2(0.0, 0.0);
            for (int r = 0; r < radix; ++r) {
                double2 w = roots[(long long)((long long)r * e0 % span) * tw_step];
                if (inverse) w.y = -w.y;
                sum = zadd(sum, zmul(a[j + r * in_step], w));
            }
            b[o] = sum;
        }
        __syncthreads();
        double2* t = a;
        a = b;
        b = t;
        ns = span;
    }
    for (int k = threadIdx.x; k < n; k += blockDim.x)
        base[(long long)k * stride] = make_double2(a[k].x * scale, a[k].y * scale);
}

// Power-of-two lengths: the same Stockham autosort with radix-4
// butterflies (after one radix-2 stage when log2 n is odd), one thread per
// butterfly and index arithmetic by shifts and masks. With span = 4 ns, the
// outputs q of input group j are X_q = sum_r t_r w_4^(r q), where
// t_r = a[j + r n/4] w_span^(r (j mod ns)) and w_span^k = roots[k n / span].
__global__ void fft_lines_pow2_kernel(double2* const* arrays, int n, int log2n, long long stride, long long dist,
                                      const double2* __restrict__ roots, int inverse, double scale) {
    extern __shared__ double2 zsm[];
    double2* a = zsm;
    double2* b = zsm + n;
    double2* base = arrays[blockIdx.y] + (long long)blockIdx.x * dist;
    for (int k = threadIdx.x; k < n; k += blockDim.x) a[k] = base[(long long)k * stride];
    __syncthreads();
    int ls = 0;  // log2 of the completed sub-transform length ns
    if (log2n & 1) {
        const int half = n >> 1;
        for (int j = threadIdx.x; j < half; j += blockDim.x) {
            const double2 x0 = a[j], x1 = a[j + half];
            b[2 * j] = make_double2(x0.x + x1.x, x0.y + x1.y);
            b[2 * j + 1] = make_double2(x0.x - x1.x, x0.y - x1.y);
        }
        __syncthreads();
        double2* t = a;
        a = b;
        b = t;
        ls = 1;
    }
    const int quarter = n >> 2;
    for (; ls < log2n; ls += 2) {
        const int ns = 1 << ls;
        const int tw_shift = log2n - ls - 2;
        for (int j = threadIdx.x; j < quarter; j += blockDim.x) {
            const int jm = j & (ns - 1);
            double2 t0 = a[j], t1 = a[j + quarter], t2 = a[j + 2 * quarter], t3 = a[j + 3 * quarter];
            if (jm) {
                double2 w1 = roots[jm << tw_shift], w2 = roots[(2 * jm) << tw_shift], w3 = roots[(3 * jm) << tw_shift];
                if (inverse) {
                    w1.y = -w1.y;
                    w2.y = -w2.y;
                    w3.y = -w3.y;
                }
                t1 = zmul(t1, w1);
                t2 = zmul(t2, w2);
                t3 = zmul(t3, w3);
            }
            const double2 s02 = make_double2(t0.x + t2.x, t0.y + t2.y), d02 = make_double2(t0.x - t2.x, t0.y - t2.y);
            const double2 s13 = make_double2(t1.x + t3.x, t1.y + t3.y), d13 = make_double2(t1.x - t3.x, t1.y - t3.y);
            // w_4 = -i forward, +i inverse: X1 = d02 + w_4 d13, X3 = d02 - w_4 d13.
            const double2 wd = inverse ? make_double2(-d13.y, d13.x) : make_double2(d13.y, -d13.x);
            const int o = ((j >> ls) << (ls + 2)) + jm;
            b[o] = make_double2(s02.x + s13.x, s02.y + s13.y);
            b[o + ns] = make_double2(d02.x + wd.x, d02.y + wd.y);
            b[o + 2 * ns] = make_double2(s02.x - s13.x, s02.y - s13.y);
            b[o + 3 * ns] = make_double2(d02.x - wd.x, d02.y - wd.y);
        }
        __syncthreads();
        double2* t = a;
        a = b;
        b = t;
    }
    for (int k = threadIdx.x; k < n; k += blockDim.x)
        base[(long long)k * stride] = make_double2(a[k].x * scale, a[k].y * scale);
}

cudaError_t launch_fft_lines(double2* const* arrays, int count, int n, long long stride, long long dist, int lines,
                             int inverse, const double2* roots, const int* factors, int nfactors, double scale,
                             cudaStream_t s) {
    const size_t smem = sizeof(double2) * 2 * (size_t)n;
    if (n >= 4 && (n & (n - 1)) == 0) {
        int log2n = 0;
        while ((1 << log2n) < n) ++log2n;
        if (smem > 48 * 1024) {
            cudaError_t e =
                cudaFuncSetAttribute(fft_lines_pow2_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess) return e;
        }
        const int threads = n / 4 < 32 ? 32 : (n / 4 > 256 ? 256 : n / 4);
        fft_lines_pow2_kernel<<<dim3(lines, count), threads, smem, s>>>(arrays, n, log2n, stride, dist, roots, inverse,
                                                                        scale);
        return cudaGetLastError();
    }
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(fft_lines_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    const int threads = n >= 256 ? 256 : (n >= 64 ? 64 : 32);
    fft_lines_kernel<<<dim3(lines, count), threads, smem, s>>>(arrays, n, stride, dist, roots, factors, nfactors,
                                                               inverse, scale);
    return cudaGetLastError();
}

// Natural FP64 spectrum -> centred FP32 state (fftshift), anchor copy and
// zero velocity for mPIE. The state row stride is M rounded up to even.
__global__ void shift_to_state_kernel(double2* const* scratch, float2* const* object, float2* const* anchor,
                                      float2* const* velocity, int m) {
    const int tile = blockIdx.y;
    const long long ms = m + (m & 1);
    const long long total = (long long)m * ms;
    const double2* src = scratch[tile];
    float2* o = object[tile];
    if (!o) return;  // a tile left out of this pass
    float2* a = anchor ? anchor[tile] : nullptr;
    float2* v = velocity ? velocity[tile] : nullptr;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
        const int r = (int)(e / ms), c = (int)(e % ms);
        float2 val = make_float2(0.f, 0.f);
        if (c < m) {
            // fftshift_copy: dst[(r + m/2) % m] = src[r]  =>  src = (dst - m/2) mod m.
            const int sr = (r + m - m / 2) % m, sc = (c + m - m / 2) % m;
            const double2 z = src[(long long)sr * m + sc];
            val = make_float2((float)z.x, (float)z.y);
        }
        o[e] = val;
        if (a) a[e] = val;
        if (v) v[e] = make_float2(0.f, 0.f);
    }
}

cudaError_t launch_shift_to_state(double2* const* scratch, float2* const* object, float2* const* anchor,
                                  float2* const* velocity, int count, int m, cudaStream_t s) {
    const long long total = (long long)m * (m + (m & 1));
    const int blocks = (int)((total + 255) / 256 < 512 ? (total + 255) / 256 : 512);
    shift_to_state_kernel<<<dim3(blocks, count), 256, 0, s>>>(scratch, object, anchor, velocity, m);
    return cudaGetLastError();
}

// Centred FP32 state -> natural FP64 scratch (ifftshift) before the inverse FFT.
__global__ void state_to_natural_kernel(const float2* const* object, double2* const* scratch, int m) {
    const int tile = blockIdx.y;
    const long long ms = m + (m & 1);
    const long long total = (long long)m * m;
    const float2* o = object[tile];
    double2* dst = scratch[tile];
    const int h = (m + 1) / 2;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
        const int r = (int)(e / m), c = (int)(e % m);
        const float2 v = o[(long long)r * ms + c];
        dst[(long long)((r + h) % m) * m + (c + h) % m] = make_double2((double)v.x, (double)v.y);
    }
}

cudaError_t launch_state_to_natural(const float2* const* object, double2* const* scratch, int count, int m,
                                    cudaStream_t s) {
    const long long total = (long long)m * m;
    const int blocks = (int)((total + 255) / 256 < 512 ? (total + 255) / 256 : 512);
    state_to_natural_kernel<<<dim3(blocks, count), 256, 0, s>>>(object, scratch, m);
    return cudaGetLastError();
}

// Complex64 rows (row stride src_stride) widened to dense complex128.
__global__ void widen_kernel(const float2* __restrict__ src, long long src_stride, int rows, int cols,
                             double2* __restrict__ dst) {
    const long long total = (long long)rows * cols;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
        const long long r = e / cols, c = e % cols;
        const float2 v = src[r * src_stride + c];
        dst[e] = make_double2((double)v.x, (double)v.y);
    }
}

cudaError_t launch_widen(const float2* src, long long src_stride, int rows, int cols, double2* dst, cudaStream_t s) {
    const long long total = (long long)rows * cols;
    if (total == 0) return cudaSuccess;
    const int blocks = (int)((total + 255) / 256 < 1024 ? (total + 255) / 256 : 1024);
    widen_kernel<<<blocks, 256, 0, s>>>(src, src_stride, rows, cols, dst);
    return cudaGetLastError();
}

// Dense complex128 rows narrowed to complex64 rows of stride dst_stride
// (checkpoint restore: the values were widened from complex64, so this is exact).
__global__ void narrow_kernel(const double2* __restrict__ src, int rows, int cols, float2* __restrict__ dst,
                              long long dst_stride) {
    // Every destination element, pad columns (c >= cols) set to zero: the
    // stencil staging reads whole column pairs.
    const long long total = (long long)rows * dst_stride;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
        const long long r = e / dst_stride, c = e % dst_stride;
        float2 out = make_float2(0.f, 0.f);
        if (c < cols) {
            const double2 v = src[r * cols + c];
            out = make_float2((float)v.x, (float)v.y);
        }
        dst[e] = out;
    }
}

cudaError_t launch_narrow(const double2* src, int rows, int cols, float2* dst, long long dst_stride, cudaStream_t s) {
    const long long total = (long long)rows * cols;
    if (total == 0) return cudaSuccess;
    const int blocks = (int)((total + 255) / 256 < 1024 ? (total + 255) / 256 : 1024);
    narrow_kernel<<<blocks, 256, 0, s>>>(src, rows, cols, dst, dst_stride);
    return cudaGetLastError();
}

// ------------------------------------------------------------------ gauge

constexpr int kGaugeThreads = 1024;

struct ArgMax {
    double weight;
    long long index;
    double2 value;
};

__device__ __forceinline__ void argmax_take(ArgMax& a, const ArgMax& b) {
    if (b.weight > a.weight || (b.weight == a.weight && b.index < a.index && b.weight > 0.0)) a = b;
}

// Deterministic block reduction of (sum complex, sum real, argmax) triples.
struct Reduction {
    double2 sum;
    double total;
    ArgMax best;
};

__device__ Reduction block_reduce(Reduction v, Reduction* scratch) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        Reduction other;
        other.sum.x = __shfl_down_sync(0xffffffffu, v.sum.x, o);
        other.sum.y = __shfl_down_sync(0xffffffffu, v.sum.y, o);
        other.total = __shfl_down_sync(0xffffffffu, v.total, o);
        other.best.weight = __shfl_down_sync(0xffffffffu, v.best.weight, o);
        other.best.index = __shfl_down_sync(0xffffffffu, v.best.index, o);
        other.best.value.x = __shfl_down_sync(0xffffffffu, v.best.value.x, o);
        other.best.value.y = __shfl_down_sync(0xffffffffu, v.best.value.y, o);
        v.sum = zadd(v.sum, other.sum);
        v.total += other.total;
        argmax_take(v.best, other.best);
    }
    if (lane == 0) scratch[warp] = v;
    __syncthreads();
    Reduction r;
    if (threadIdx.x == 0) {
        r = scratch[0];
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) {
            r.sum = zadd(r.sum, scratch[w].sum);
            r.total += scratch[w].total;
            argmax_take(r.best, scratch[w].best);
        }
        scratch[0] = r;
    }
    __syncthreads();
    r = scratch[0];
    __syncthreads();
    return r;
}

__device__ __forceinline__ Reduction empty_reduction() {
    Reduction r;
    r.sum = make_double2(0.0, 0.0);
    r.total = 0.0;
    r.best.weight = 0.0;
    r.best.index = 0x7fffffffffffffffLL;
    r.best.value = make_double2(0.0, 0.0);
    return r;
}

__device__ __forceinline__ double2 load_z(const float2* p) {
    const float2 v = *p;
    return make_double2((double)v.x, (double)v.y);
}

__device__ __forceinline__ void store_z(float2* p, double2 z) { *p = make_float2((float)z.x, (float)z.y); }

// relative_phase_slope (src/algorithms/gauge.rs:75-130).
__device__ double phase_slope(const GaugeTile& T, int n, bool axis_row, double tol, Reduction* scratch) {
    Reduction acc = empty_reduction();
    const int rows = axis_row ? n - 1 : n, cols = axis_row ? n : n - 1;
    for (int e = threadIdx.x; e < rows * cols; e += blockDim.x) {
        const int r = e / cols, c = e % cols;
        const int cur = r * n + c;
        const int nxt = axis_row ? (r + 1) * n + c : cur + 1;
        if (T.support[cur] == 0 || T.support[nxt] == 0) continue;
        const double2 ce = zmul(load_z(T.pupil + nxt), zconj(load_z(T.pupil + cur)));
        const double2 re = zmul(T.reference[nxt], zconj(T.reference[cur]));
        const double2 contribution = zmul(ce, zconj(re));
        const double weight = hypot(contribution.x, contribution.y);
        if (!isfinite(weight)) continue;
        acc.sum = zadd(acc.sum, contribution);
        acc.total += weight;
        ArgMax b = {weight, (long long)cur, contribution};
        argmax_take(acc.best, b);
    }
    Reduction r = block_reduce(acc, scratch);
    if (r.total == 0.0) return 0.0;
    if (hypot(r.sum.x, r.sum.y) > tol * r.total) return atan2(r.sum.y, r.sum.x);
    if (r.best.weight > 0.0) return atan2(r.best.value.y, r.best.value.x);
    return 0.0;
}

__global__ void __launch_bounds__(kGaugeThreads) gauge_kernel(const GaugeTile* tiles, int n, int m) {
    __shared__ Reduction scratch[kGaugeThreads / 32];
    __shared__ int s_fail;
    const GaugeTile T = tiles[blockIdx.x];
    const long long ms = m + (m & 1);
    if (threadIdx.x == 0) s_fail = 0;
    // support count
    Reduction cnt = empty_reduction();
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) cnt.total += T.support[e] != 0 ? 1.0 : 0.0;
    cnt = block_reduce(cnt, scratch);
    const double support_count = cnt.total;
    if (support_count == 0.0) {
        if (threadIdx.x == 0) atomicOr(T.status, 8);
        return;
    }
    const double tol = 64.0 * 2.220446049250313e-16 * support_count;
    const double row_slope = T.row_exact ? phase_slope(T, n, true, tol, scratch) : 0.0;
    const double col_slope = T.col_exact ? phase_slope(T, n, false, tol, scratch) : 0.0;
    if (fabs(row_slope) > tol || fabs(col_slope) > tol) {
        for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
            const double y = (double)(e / n) - (double)(n / 2), x = (double)(e % n) - (double)(n / 2);
            double sn, cs;
            sincos(-(row_slope * y + col_slope * x), &sn, &cs);
            store_z(T.pupil + e, zmul(load_z(T.pupil + e), make_double2(cs, sn)));
        }
        for (long long e = threadIdx.x; e < (long long)m * m; e += blockDim.x) {
            const int r = (int)(e / m), c = (int)(e % m);
            const double y = (double)r - (double)(m / 2), x = (double)c - (double)(m / 2);
            double sn, cs;
            sincos(row_slope * y + col_slope * x, &sn, &cs);
            float2* p = T.object + (long long)r * ms + c;
            store_z(p, zmul(load_z(p), make_double2(cs, sn)));
        }
        __syncthreads();
    }
    // normalize_pupil_scale_and_phase (src/algorithms/gauge.rs:158-240)
    Reduction energy = empty_reduction();
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
        if (T.support[e] == 0) continue;
        energy.sum.x += zabs2(T.reference[e]);
        energy.sum.y += zabs2(load_z(T.pupil + e));
    }
    energy = block_reduce(energy, scratch);
    const double ref_energy = energy.sum.x, cur_energy = energy.sum.y;
    if (!isfinite(ref_energy) || ref_energy <= 0.0 || !isfinite(cur_energy) || cur_energy <= 0.0) {
        if (threadIdx.x == 0) atomicOr(T.status, 8);
        return;
    }
    const double computed = sqrt(ref_energy / cur_energy);
    const double scale = fabs(computed - 1.0) <= tol ? 1.0 : computed;
    Reduction overlap = empty_reduction();
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
        if (T.support[e] == 0) continue;
        const double2 contribution = zmul(zconj(T.reference[e]), load_z(T.pupil + e));
        const double weight = hypot(contribution.x, contribution.y);
        overlap.sum = zadd(overlap.sum, contribution);
        overlap.total += weight;
        ArgMax b = {weight, (long long)e, contribution};
        argmax_take(overlap.best, b);
    }
    overlap = block_reduce(overlap, scratch);
    double phase;
    if (overlap.total > 0.0 && hypot(overlap.sum.x, overlap.sum.y) > tol * overlap.total)
        phase = atan2(overlap.sum.y, overlap.sum.x);
    else if (overlap.best.weight > 0.0)
        phase = atan2(overlap.best.value.y, overlap.best.value.x);
    else {
        if (threadIdx.x == 0) atomicOr(T.status, 8);
        return;
    }
    if (fabs(phase) <= tol) phase = 0.0;
    double sp, cp;
    sincos(-phase, &sp, &cp);
    const double2 pupil_factor = make_double2(scale * cp, scale * sp);
    if (!(pupil_factor.x == 1.0 && pupil_factor.y == 0.0)) {
        const double d = zabs2(pupil_factor);
        const double2 object_factor = make_double2(pupil_factor.x / d, -pupil_factor.y / d);
        for (int e = threadIdx.x; e < n * n; e += blockDim.x)
            store_z(T.pupil + e, zmul(load_z(T.pupil + e), pupil_factor));
        for (long long e = threadIdx.x; e < (long long)m * m; e += blockDim.x) {
            float2* p = T.object + (e / m) * ms + (e % m);
            store_z(p, zmul(load_z(p), object_factor));
        }
        __syncthreads();
    }
    // normalize_object_phase (src/algorithms/gauge.rs:242-282)
    Reduction strongest = empty_reduction();
    for (long long e = threadIdx.x; e < (long long)m * m; e += blockDim.x) {
        const double2 v = load_z(T.object + (e / m) * ms + (e % m));
        if (!isfinite(v.x) || !isfinite(v.y)) s_fail = 1;
        ArgMax b = {hypot(v.x, v.y), e, v};
        argmax_take(strongest.best, b);
    }
    strongest = block_reduce(strongest, scratch);
    if (s_fail) {
        if (threadIdx.x == 0) atomicOr(T.status, 8);
        return;
    }
    if (strongest.best.weight == 0.0) return;
    const double2 dc = load_z(T.object + (long long)(m / 2) * ms + m / 2);
    const double2 anchor = hypot(dc.x, dc.y) > tol * strongest.best.weight ? dc : strongest.best.value;
    const double object_phase = atan2(anchor.y, anchor.x);
    if (fabs(object_phase) <= tol) return;
    double so, co;
    sincos(-object_phase, &so, &co);
    const double2 correction = make_double2(co, so);
    for (long long e = threadIdx.x; e < (long long)m * m; e += blockDim.x) {
        float2* p = T.object + (e / m) * ms + (e % m);
        store_z(p, zmul(load_z(p), correction));
    }
}

cudaError_t launch_gauge(const GaugeTile* tiles, int count, int n, int m, cudaStream_t s) {
    gauge_kernel<<<count, kGaugeThreads, 0, s>>>(tiles, n, m);
    return cudaGetLastError();
}

// ------------------------------------------------------- GD regularisers

__device__ __forceinline__ double2 zsub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double znorm2(double2 a) { return a.x * a.x + a.y * a.y; }

// Normalised forward differences of pixel (r, c) for the smoothed TV: the
// horizontal and vertical differences over sqrt(|dh|^2 + |dv|^2 + eps^2),
// each zero where the neighbour is outside the grid.
__device__ __forceinline__ void tv_terms(const double2* __restrict__ v, int m, int r, int c, double eps2, double2& qh,
                                         double2& qv) {
    const double2 x = v[(long long)r * m + c];
    const bool has_h = c + 1 < m, has_v = r + 1 < m;
    const double2 dh = has_h ? zsub(v[(long long)r * m + c + 1], x) : make_double2(0.0, 0.0);
    const double2 dv = has_v ? zsub(v[(long long)(r + 1) * m + c], x) : make_double2(0.0, 0.0);
    const double inv = 1.0 / sqrt((has_h ? znorm2(dh) : 0.0) + (has_v ? znorm2(dv) : 0.0) + eps2);
    qh = make_double2(dh.x * inv, dh.y * inv);
    qv = make_double2(dv.x * inv, dv.y * inv);
}

// apply_complex_tv_step (src/algorithms/regularization.rs:5-48) as a
// gather: the gradient at p is -(qh(p) + qv(p)) + qh(left) + qv(above).
__global__ void object_tv_kernel(const RegularTile* tiles, int m, double epsilon) {
    const RegularTile& T = tiles[blockIdx.y];
    const double eps2 = epsilon * epsilon;
    const long long total = (long long)m * m;
    bool bad = false;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
        const int r = (int)(e / m), c = (int)(e % m);
        double2 qh, qv, g;
        tv_terms(T.src, m, r, c, eps2, qh, qv);
        g = make_double2(-(qh.x + qv.x), -(qh.y + qv.y));
        if (c >= 1) {
            tv_terms(T.src, m, r, c - 1, eps2, qh, qv);
            g.x += qh.x;
            g.y += qh.y;
        }
        if (r >= 1) {
            tv_terms(T.src, m, r - 1, c, eps2, qh, qv);
            g.x += qv.x;
            g.y += qv.y;
        }
        const double2 x = T.src[e];
        const double2 y = make_double2(x.x - T.weight * g.x, x.y - T.weight * g.y);
        bad |= !isfinite(y.x) || !isfinite(y.y);
        T.dst[e] = y;
    }
    if (bad) atomicOr(T.status, 128);
}

cudaError_t launch_object_tv(const RegularTile* tiles, int count, int m, double epsilon, cudaStream_t s) {
    const long long total = (long long)m * m;
    const int blocks = (int)((total + 255) / 256 < 1024 ? (total + 255) / 256 : 1024);
    object_tv_kernel<<<dim3(blocks, count), 256, 0, s>>>(tiles, m, epsilon);
    return cudaGetLastError();
}

// apply_quadratic_smoothing_step (src/algorithms/regularization.rs:50-80)
// into the scratch, then the support, then back into the pupil.
__global__ void pupil_smoothing_kernel(const RegularTile* tiles, int n, int constrain) {
    const RegularTile& T = tiles[blockIdx.y];
    const long long total = (long long)n * n;
    bool bad = false;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
        const int r = (int)(e / n), c = (int)(e % n);
        const float2 xf = T.pupil[e];
        const double2 x = make_double2(xf.x, xf.y);
        // The reference's scatter sums to grad = -2 * sum over the grid
        // neighbours of (neighbour - x).
        double2 g = make_double2(0.0, 0.0);
        auto add = [&](long long q) {
            const float2 yf = T.pupil[q];
            g.x -= 2.0 * ((double)yf.x - x.x);
            g.y -= 2.0 * ((double)yf.y - x.y);
        };
        if (c + 1 < n) add(e + 1);
        if (r + 1 < n) add(e + n);
        if (c >= 1) add(e - 1);
        if (r >= 1) add(e - n);
        double2 y = make_double2(x.x - T.weight * g.x, x.y - T.weight * g.y);
        bad |= !isfinite(y.x) || !isfinite(y.y);
        if (constrain && T.support[e] == 0) y = make_double2(0.0, 0.0);
        T.pupil_scratch[e] = make_float2((float)y.x, (float)y.y);
    }
    if (bad) atomicOr(T.status, 128);
}

__global__ void pupil_copy_kernel(const RegularTile* tiles, int n) {
    const RegularTile& T = tiles[blockIdx.y];
    const long long total = (long long)n * n;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x)
        T.pupil[e] = T.pupil_scratch[e];
}

cudaError_t launch_pupil_smoothing(const RegularTile* tiles, int count, int n, int constrain, cudaStream_t s) {
    const long long total = (long long)n * n;
    const int blocks = (int)((total + 255) / 256 < 256 ? (total + 255) / 256 : 256);
    pupil_smoothing_kernel<<<dim3(blocks, count), 256, 0, s>>>(tiles, n, constrain);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    pupil_copy_kernel<<<dim3(blocks, count), 256, 0, s>>>(tiles, n);
    return cudaGetLastError();
}

// ------------------------------------------------ illumination recovery

// Natural detector (y, x) -> engine layout index of an n x n frame (the
// frame engine's CTA-row and digit permutation).
__device__ int engine_index(int n, int y, int x) {
    const int r = n >= 128 ? 16 : 32, c = n / r, na = n >= 128 ? 16 : 8, nb = n / na;
    return ((y % c) * r + y / c) * n + nb * (x % na) + x / na;
}

__device__ bool task_frame(const IlluminationTile& T, const IlluminationTask& task, int& f) {
    if (task.position >= T.frame_count) return false;
    f = T.order ? T.order[task.position] : task.position;
    return T.params[f].weight != 0.f;
}

// compute_source_field (src/algorithms/gradient_descent.rs:1184-1213) for
// evaluation e of a task: the bilinear FP64 patch of the state at the
// offset (compiled + correction, +-d on one axis for e > 0) times the
// pupil, ifftshifted into the inverse FFT's input. blockIdx.y = task * 5 + e.
__global__ void illumination_fields_kernel(const IlluminationParams P) {
    const int task_index = blockIdx.y / 5, e = blockIdx.y % 5;
    const IlluminationTask task = P.tasks[task_index];
    const IlluminationTile& T = P.tiles[task.tile];
    const int n = P.n;
    double2* out = P.fields + (size_t)blockIdx.y * n * n;
    int f = 0;
    bool ok = task_frame(T, task, f);
    long long lr = 0, lc = 0;
    double fr = 0.0, fc = 0.0;
    if (ok) {
        const double d = (e == 2 || e == 4) ? -P.distance : P.distance;
        const double orow = T.offset[2 * f] + T.correction[2 * f] + (e == 1 || e == 2 ? d : 0.0);
        const double ocol = T.offset[2 * f + 1] + T.correction[2 * f + 1] + (e >= 3 ? d : 0.0);
        ok = offset_axis(T.start[2 * f], n, T.M, orow, lr, fr) && offset_axis(T.start[2 * f + 1], n, T.M, ocol, lc, fc);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) P.valid[blockIdx.y] = ok ? 1 : 0;
    if (!ok) {
        // Skipped evaluation: a defined (zero) field through the FFT.
        for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n * n; p += gridDim.x * blockDim.x)
            out[p] = make_double2(0.0, 0.0);
        return;
    }
    const long long ostride = T.M + (T.M & 1);
    const int half = n / 2;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n * n; p += gridDim.x * blockDim.x) {
        const int i = p / n, j = p % n;  // centred patch coordinates
        const float2* row0 = T.object + (lr + i) * ostride + lc + j;
        const float2 a = row0[0];
        double re = (1.0 - fr) * (1.0 - fc) * a.x, im = (1.0 - fr) * (1.0 - fc) * a.y;
        if (fc > 0.0) {
            const float2 b = row0[1];
            re += (1.0 - fr) * fc * b.x;
            im += (1.0 - fr) * fc * b.y;
        }
        if (fr > 0.0) {
            const float2 c = row0[ostride];
            re += fr * (1.0 - fc) * c.x;
            im += fr * (1.0 - fc) * c.y;
            if (fc > 0.0) {
                const float2 g = row0[ostride + 1];
                re += fr * fc * g.x;
                im += fr * fc * g.y;
            }
        }
        const float2 pu = T.pupil[p];
        const double2 v = make_double2(re * pu.x - im * pu.y, re * pu.y + im * pu.x);
        out[(size_t)((i + half) % n) * n + (j + half) % n] = v;
    }
}

cudaError_t launch_illumination_fields(const IlluminationParams& p, int tasks, cudaStream_t s) {
    if (tasks <= 0) return cudaSuccess;
    const int blocks = (p.n * p.n + 255) / 256 < 64 ? (p.n * p.n + 255) / 256 : 64;
    illumination_fields_kernel<<<dim3(blocks, tasks * 5), 256, 0, s>>>(p);
    return cudaGetLastError();
}

// descent_factor and descent_curvature (src/algorithms/gradient_descent.rs:
// 1167-1178, 1340-1360) in FP64.
__device__ double gd_factor(double predicted, double measured, int loss, double eps) {
    switch (loss) {
        case 0: return 1.0 - sqrt(fmax(measured, 0.0)) / sqrt(fmax(predicted, eps));
        case 1: return 2.0 * (predicted - measured);
        case 2: return 1.0 - fmax(measured, 0.0) / fmax(predicted, eps);
        default: {
            const double pa = sqrt(fmax(predicted, eps));
            return fmin(fmax(pa - sqrt(fmax(measured, 0.0)), -1.0), 1.0) / (2.0 * pa);
        }
    }
}

__device__ double gd_curvature(double predicted, double factor, int loss, double eps) {
    const double mean = fmax(predicted, eps);
    switch (loss) {
        case 0: return 0.5 / mean;
        case 1: return 2.0;
        case 2: return 1.0 / mean;
        default: return fabs(factor * 2.0 * sqrt(mean)) < 1.0 ? 0.25 / mean : eps;
    }
}

// illumination_axis_gradient (src/algorithms/gradient_descent.rs:1272-1338):
// block (b, task) takes pixel slice b of the task's frame; over the pixels
// the gradient step retains (unmasked, no truncation), the loss derivative at
// the current offset times central (or, at the grid edge, one-sided)
// differences of the intensity, and the Gauss-Newton curvature times their
// squares, per axis, summed in a fixed order into the slice's partials.
constexpr int kIllumReduceThreads = 256;

__global__ void __launch_bounds__(kIllumReduceThreads) illumination_reduce_kernel(const IlluminationParams P) {
    __shared__ double red[kIllumReduceThreads / 32][4];
    const IlluminationTask task = P.tasks[blockIdx.y];
    const IlluminationTile& T = P.tiles[task.tile];
    int f = 0;
    if (!task_frame(T, task, f)) return;
    const int n = P.n;
    const size_t n2 = (size_t)n * n;
    const int* valid = P.valid + (size_t)blockIdx.y * 5;
    const double2* field = P.fields + (size_t)blockIdx.y * 5 * n2;
    const int slice = (int)((n2 + kIlluminationBlocks - 1) / kIlluminationBlocks);
    const int p_begin = blockIdx.x * slice, p_end = min((int)n2, p_begin + slice);
    const bool ok[5] = {valid[0] != 0, valid[1] != 0, valid[2] != 0, valid[3] != 0, valid[4] != 0};
    // The current stencil is always inside the grid; were it not, the slice
    // would add nothing.
    const int p_stop = ok[0] ? p_end : p_begin;
    const double gain = (double)T.params[f].gain;
    const double d = P.distance;
    const size_t frame_base = (size_t)f * n2;
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    for (int p = p_begin + threadIdx.x; p < p_stop; p += blockDim.x) {
        const int idx = engine_index(n, p / n, p % n);
        const double m = (double)T.meas[frame_base + idx];
        bool keep;
        double target;
        if (T.amplitude) {
            keep = m >= 0.0;
            target = m * m;
        } else {
            keep = !T.masks || T.masks[frame_base + idx] != 0;
            const double bg = T.background ? (double)T.background[(size_t)f * T.background_stride + idx] : 0.0;
            target = fmax((m - bg) / gain, 0.0);
        }
        if (!keep) continue;
        const double2 f0 = field[p];
        const double pred = f0.x * f0.x + f0.y * f0.y;
        const double factor = gd_factor(pred, target, P.loss, P.epsilon);
        const double curv = gd_curvature(pred, factor, P.loss, P.epsilon);
#pragma unroll
        for (int a = 0; a < 2; ++a) {
            const bool plus = ok[1 + 2 * a], minus = ok[2 + 2 * a];
            if (!plus && !minus) continue;
            const double2 fp = field[(size_t)(1 + 2 * a) * n2 + p];
            const double2 fm = field[(size_t)(2 + 2 * a) * n2 + p];
            const double ip = fp.x * fp.x + fp.y * fp.y, im = fm.x * fm.x + fm.y * fm.y;
            const double der = plus && minus ? (ip - im) / (2.0 * d) : plus ? (ip - pred) / d : (pred - im) / d;
            acc[a] += factor * der;
            acc[2 + a] += curv * der * der;
        }
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        double v = acc[a];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) red[warp][a] = v;
    }
    __syncthreads();
    if (threadIdx.x < 4) {
        double total = 0.0;
        for (int w = 0; w < kIllumReduceThreads / 32; ++w) total += red[w][threadIdx.x];
        T.partials[((size_t)f * kIlluminationBlocks + blockIdx.x) * 4 + threadIdx.x] = total;
    }
}

cudaError_t launch_illumination_reduce(const IlluminationParams& p, int tasks, cudaStream_t s) {
    if (tasks <= 0) return cudaSuccess;
    illumination_reduce_kernel<<<dim3(kIlluminationBlocks, tasks), kIllumReduceThreads, 0, s>>>(p);
    return cudaGetLastError();
}

// apply_illumination_update (src/algorithms/gradient_descent.rs:1044-1089),
// one thread per task of the batch: the frame's sums times weight / unmasked
// pixels, a bounded Gauss-Newton step kept only while the corrected stencil
// stays inside the grid, and then the frame's stencil fields follow it.
__global__ void illumination_update_kernel(const IlluminationTile* tiles, const IlluminationTask* tasks, int count,
                                           int n, double step, double bound, double epsilon) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= count) return;
    const IlluminationTask task = tasks[t];
    const IlluminationTile& T = tiles[task.tile];
    int f = 0;
    if (!task_frame(T, task, f)) return;
    FrameParam fp = T.params[f];
    if (fp.loss_scale == 0.0) return;
    double sum[4] = {0.0, 0.0, 0.0, 0.0};
    for (int b = 0; b < kIlluminationBlocks; ++b)
        for (int a = 0; a < 4; ++a) sum[a] += T.partials[((size_t)f * kIlluminationBlocks + b) * 4 + a];
    for (int a = 0; a < 4; ++a) sum[a] *= fp.loss_scale;
    if (!isfinite(sum[0]) || !isfinite(sum[1]) || !isfinite(sum[2]) || !isfinite(sum[3]) || sum[2] < 0.0 ||
        sum[3] < 0.0) {
        atomicOr(T.status, 256);
        return;
    }
    const double cr = fmin(fmax(T.correction[2 * f] - step * sum[0] / (sum[2] + epsilon), -bound), bound);
    const double cc = fmin(fmax(T.correction[2 * f + 1] - step * sum[1] / (sum[3] + epsilon), -bound), bound);
    if (offset_frame_param(T.start[2 * f], T.start[2 * f + 1], T.offset[2 * f] + cr, T.offset[2 * f + 1] + cc, n,
                           T.M, fp)) {
        T.correction[2 * f] = cr;
        T.correction[2 * f + 1] = cc;
        T.params[f] = fp;
    }
}

cudaError_t launch_illumination_update(const IlluminationTile* tiles, const IlluminationTask* tasks, int count,
                                       int n, double step, double bound, double epsilon, cudaStream_t s) {
    if (count <= 0) return cudaSuccess;
    illumination_update_kernel<<<(count + 127) / 128, 128, 0, s>>>(tiles, tasks, count, n, step, bound, epsilon);
    return cudaGetLastError();
}

}  // namespace fpm
