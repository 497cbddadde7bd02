// Frame engine: the per-frame FPM update of src/algorithms/common.rs:57-306
// (AP / FPIE / mPIE / EPRY) and src/algorithms/gradient_descent.rs:405-671
// (batch-1 Wirtinger gradient) for many independent tiles in one launch.
//
// One thread-block cluster owns one tile for the whole launch and walks its
// frames in the reference's exact sequential order. A cluster has C = N/32
// CTAs; CTA c holds 32 rows of the N x N detector field in shared memory:
// the centred patch rows [32c, 32c + 32), which are natural rows of block
// c ^ (C/2) because fftshift moves whole 32-row blocks when C >= 2. Per frame:
//
//   S0  stage the bilinear stencil of the object spectrum (33 x (N+1)) in smem
//   P1  gather patch * pupil (ifftshifted), row IFFT step A (radix NA)
//   P2  row IFFT step C (radix NB)                     -> cluster barrier
//   P3  column IFFT across the cluster (radix C, DSMEM)-> cluster barrier
//   P4  column IFFT (radix 32, registers), |psi|^2, projection or descent
//       factor, column FFT (radix 32)                  -> cluster barrier
//   P5  column FFT across the cluster (radix C, DSMEM) -> cluster barrier
//   P6  row FFT step C'                                -> block barrier
//   P7  row FFT step A', fftshift, correction U, EPRY pupil update
//   P8  exact bilinear adjoint of U added into the object (src/model/crop.rs:188-255)
//
// The IFFT leaves its output in digit-permuted order and the FFT consumes that
// order, so no bit-reversal or transpose pass exists. HBM traffic per frame is
// the stencil read and write plus the measurement frame; the field never
// leaves the cluster. Complex arithmetic is FP32; loss sums are FP64.
#pragma once

#include <cooperative_groups.h>

#include "fpm_common.cuh"
#include "kernels.h"

namespace cg = cooperative_groups;

namespace fpm {

template <int N_>
struct Cfg {
    static constexpr int N = N_;
    // Field rows per CTA. 128- and 256-point tiles use 16-row CTAs (8- and
    // 16-CTA clusters): about 56 KB and 108 KB of shared memory each, so four
    // or two tiles' CTAs share an SM and hide each other's barrier and
    // exchange latency.
    static constexpr int R = N >= 128 ? 16 : 32;
    static constexpr int C = N / R;         // CTAs per cluster
    static constexpr int NA = N >= 128 ? 16 : 8;
    static constexpr int NB = N / NA;
    // Padded field row stride (float2): one pad after each group of NB,
    // stride chosen so that half-warps spanning two rows hit disjoint banks.
    static constexpr int RS = N == 32 ? 40 : N == 64 ? 72 : N == 128 ? 152 : 272;
    static constexpr int ORS = N + 2;       // staged stencil row: N + 2 columns from an even origin
    // P4 column transforms: R = 32 splits each column over two threads
    // (lanes l, l ^ 16); R = 16 gives each column one thread.
    static constexpr int THREADS = R == 32 ? 2 * N : N;
    static constexpr int WARPS = THREADS / 32;
    // Resident CTAs per SM that shared memory allows; registers are capped to match.
    static constexpr int MIN_BLOCKS = N == 256 ? 2 : N == 128 ? 4 : N == 64 ? 4 : 7;
    static constexpr int TW = 256 / N;      // w_N^k = w_256^(k * TW)
    static constexpr int FIELD = (R + 1) * RS;  // raw row 0: halo U row from the previous CTA
    static constexpr int STAGE = (R + 1) * ORS;
    static constexpr int PSLAB = R * N;     // this CTA's R centred pupil rows
    // + per-warp FP64 loss partials and the EPRY per-warp / per-CTA maxima.
    static constexpr int SMEM_BYTES = (FIELD + STAGE + PSLAB + 256) * 8 + (WARPS + 4) * 8 + (2 * WARPS + 2) * 4;
    static constexpr int T1 = R * NB / THREADS;      // P1 / P7 tasks per thread
    static constexpr int T2 = R * NA / THREADS;      // P2 / P6 tasks per thread
    static constexpr int TX = (R / C) * N / THREADS; // P3 / P5 tasks per thread
    static constexpr int PAIRS = N / 2 + 1;          // 16-byte pairs per staged row
    static_assert(N == 32 || N == 64 || N == 128 || N == 256, "unsupported tile size");
    static_assert(RS >= N + NA && RS % 2 == 0, "row stride");
    static_assert(R % C == 0 && (R == 32 || R == 16) && (C == 1 || R * C == N), "cluster split");
    static_assert(T1 * THREADS == R * NB && T2 * THREADS == R * NA && TX * THREADS == (R / C) * N, "tasks");
    // Dynamic + static (descriptors, about 256 B) + 1 KB reserved per CTA.
    // Dynamic + static (tile and step descriptors, at most those of the
    // spectral family) + the 1 KB the SM reserves per CTA, times the CTAs per SM.
    static_assert((SMEM_BYTES + sizeof(TileDesc) + 2 * sizeof(SpectralStep) + 1024) * MIN_BLOCKS <= 233472,
                  "shared memory");
};

template <class K>
FPM_DEVICE int phys(int q) { return q + q / K::NB; }

// Centred patch row held by local row l of CTA c.
template <class K>
FPM_DEVICE int centred_row(int c, int l) {
    if constexpr (K::C == 1) return (l + K::N / 2) & (K::N - 1);
    else return c * K::R + l;
}

template <class K>
FPM_DEVICE void cluster_barrier() {
    if constexpr (K::C == 1) {
        __syncthreads();
    } else {
        cg::this_cluster().sync();
    }
}

// Bilinear sample at centred (il, j) of the staged stencil; `s` already
// includes the odd-origin offset of the staged rows.
FPM_DEVICE float2 patch_at(const float2* __restrict__ s, int ors, int il, int j, const FrameParam& fp) {
    const float2* r0 = s + il * ors + j;
    const float2* r1 = r0 + ors;
    float2 p = cscale(r0[0], fp.w00);
    p = cfma(fp.w01, r0[1], p);
    p = cfma(fp.w10, r1[0], p);
    p = cfma(fp.w11, r1[1], p);
    return p;
}

// point_loss (src/algorithms/objective.rs:47-71) in FP32. LOSS >= 0 fixes
// the loss at compile time; LOSS < 0 reads `loss` at run time.
template <int LOSS>
FPM_DEVICE float point_loss(float predicted, float measured, int runtime_loss) {
    switch (LOSS >= 0 ? LOSS : runtime_loss) {
        case 0: {
            float r = sqrtf(fmaxf(predicted, 0.f)) - sqrtf(fmaxf(measured, 0.f));
            return r * r;
        }
        case 1: {
            float r = predicted - measured;
            return r * r;
        }
        case 2: {
            float mean = fmaxf(predicted, 1e-12f);
            return mean - fmaxf(measured, 0.f) * logf(mean);
        }
        default: {
            float r = sqrtf(fmaxf(predicted, 0.f)) - sqrtf(fmaxf(measured, 0.f));
            float a = fabsf(r);
            return a <= 1.f ? 0.5f * r * r : a - 0.5f;
        }
    }
}

// descent_factor (src/algorithms/gradient_descent.rs:1167-1178) in FP32.
template <int LOSS>
FPM_DEVICE float descent_factor(float predicted, float measured, int runtime_loss, float eps) {
    switch (LOSS >= 0 ? LOSS : runtime_loss) {
        case 0:
            return 1.f - sqrtf(fmaxf(measured, 0.f)) * rsqrtf(fmaxf(predicted, eps));
        case 1:
            return 2.f * (predicted - measured);
        case 2:
            return 1.f - fmaxf(measured, 0.f) / fmaxf(predicted, eps);
        default: {
            float pa = sqrtf(fmaxf(predicted, eps));
            float r = fminf(fmaxf(pa - sqrtf(fmaxf(measured, 0.f)), -1.f), 1.f);
            return r / (2.f * pa);
        }
    }
}

// S0: asynchronous copy of the stencil rows [i_lo, i_lo + 32] x columns
// [lower_col - odd, lower_col - odd + N + 2) into shared memory. Every copy
// starts on an even column (16-byte aligned: the object row stride is even);
// bytes beyond the grid are zero-filled and never read from global memory.
template <class K, bool WAIT = true>
FPM_DEVICE void stage_object(float2* __restrict__ osm, const float2* __restrict__ object, int M, long long ostride,
                             const FrameParam& fp, int i_lo, int row_lo, int row_hi) {
    const int c0 = fp.lower_col & ~1;
    // Staged row r serves patch rows i_lo + r (and i_lo + r - 1): rows outside
    // [row_lo, row_hi + 1] are never read.
    const int r_begin = max(row_lo - i_lo, 0), r_end = min(row_hi + 1 - i_lo, K::R);
    if (r_begin > r_end) return;
    const int count = (r_end - r_begin + 1) * K::PAIRS;
    for (int e = threadIdx.x; e < count; e += K::THREADS) {
        const int r = r_begin + e / K::PAIRS, t = e % K::PAIRS;
        const int gr = fp.lower_row + i_lo + r;
        const int col = c0 + 2 * t;
        int bytes = 0;
        if (gr < M) bytes = M - col >= 2 ? 16 : (M - col == 1 ? 8 : 0);
        const float2* src = bytes ? object + (long long)gr * ostride + col : object;
        cp_async16(osm + r * K::ORS + 2 * t, src, bytes);
    }
    if constexpr (WAIT) cp_async_wait_all();
}

// P1 + P2: patch * pupil, ifftshift, row inverse FFT into the field slab.
// Tracks maxima of |patch|^2 and |P|^2 for EPRY.
template <class K, bool TRACK_MAX>
FPM_DEVICE void rows_inverse(float2* __restrict__ fld, const float2* __restrict__ ostage, const float2* __restrict__ tw,
                             const float2* __restrict__ pslab, const FrameParam& fp, int c, int i_lo, int row_lo,
                             int row_hi, float& max_obj, float& max_pup) {
    constexpr int N = K::N, NA = K::NA, NB = K::NB;
#pragma unroll 1
    for (int t = 0; t < K::T1; ++t) {
        const int task = threadIdx.x + t * K::THREADS;
        const int l = task / NB, nb = task % NB;
        const int i = centred_row<K>(c, l);
        if (i < row_lo || i > row_hi) continue;
        const int il = i - i_lo;
        float2 v[NA];
#pragma unroll
        for (int na = 0; na < NA; ++na) {
            const int j = (NB * na + nb + N / 2) & (N - 1);
            const float2 pt = patch_at(ostage, K::ORS, il, j, fp);
            const float2 pv = pslab[il * N + j];
            if (TRACK_MAX) {
                max_obj = fmaxf(max_obj, cnorm2(pt));
                max_pup = fmaxf(max_pup, cnorm2(pv));
            }
            v[na] = cmul(pt, pv);
        }
        dft_reg<NA, true>(v);
        float2* row = fld + l * K::RS;
#pragma unroll
        for (int ka = 0; ka < NA; ++ka) row[phys<K>(NB * ka + nb)] = twiddle_smem<true>(v[ka], tw, nb * ka * K::TW);
    }
    __syncthreads();
#pragma unroll 1
    for (int t = 0; t < K::T2; ++t) {
        const int task = threadIdx.x + t * K::THREADS;
        const int l = task / NA, ka = task % NA;
        const int i = centred_row<K>(c, l);
        float2* g = fld + l * K::RS + ka * (NB + 1);
        if (i < row_lo || i > row_hi) {
            // A cluster's radix-C step substitutes zeros for such rows; a
            // single CTA's column transform reads the slab directly.
            if constexpr (K::C == 1) {
#pragma unroll
                for (int kb = 0; kb < NB; ++kb) g[kb] = make_float2(0.f, 0.f);
            }
            continue;
        }
        float2 v[NB];
#pragma unroll
        for (int kb = 0; kb < NB; ++kb) v[kb] = g[kb];
        dft_reg<NB, true>(v);
#pragma unroll
        for (int kb = 0; kb < NB; ++kb) g[kb] = v[kb];
    }
}

// P3: radix-C column step across the cluster (inverse direction): per task,
// C remote loads, one radix-C DFT and C remote stores, through explicit
// cluster-shared addresses (mapa + ld/st.shared::cluster).
template <class K>
FPM_DEVICE void columns_cross_inverse(float2* __restrict__ fld, const float2* __restrict__ tw, int c, int row_lo,
                                      int row_hi) {
    if constexpr (K::C > 1) {
        constexpr int C = K::C, N = K::N, ROWS = K::R / C;
        unsigned base[C];
#pragma unroll
        for (int r = 0; r < C; ++r) base[r] = dsmem_address(fld, r);
#pragma unroll 1
        for (int t = 0; t < K::TX; ++t) {
            const int task = threadIdx.x + t * K::THREADS;
            const int l = c * ROWS + task / N;
            const unsigned off = 8u * (unsigned)(l * K::RS + phys<K>(task % N));
            float2 v[C];
#pragma unroll
            for (int nc = 0; nc < C; ++nc) {
                // Natural block nc lives in CTA nc ^ (C / 2) as centred rows (nc ^ (C / 2)) * R + l.
                const int i = (nc ^ (C / 2)) * K::R + l;
                v[nc] = i >= row_lo && i <= row_hi ? dsmem_load(base[nc ^ (C / 2)] + off) : make_float2(0.f, 0.f);
            }
            dft_reg<C, true>(v);
#pragma unroll
            for (int k1 = 0; k1 < C; ++k1) dsmem_store(base[k1] + off, twiddle_smem<true>(v[k1], tw, l * k1 * K::TW));
        }
    }
}

// P5: radix-C column step across the cluster (forward direction); output
// block j1 goes to the CTA holding natural rows of block j1.
template <class K>
FPM_DEVICE void columns_cross_forward(float2* __restrict__ fld, int c, int row_lo, int row_hi) {
    if constexpr (K::C > 1) {
        constexpr int C = K::C, N = K::N, ROWS = K::R / C;
        unsigned base[C];
#pragma unroll
        for (int r = 0; r < C; ++r) base[r] = dsmem_address(fld, r);
#pragma unroll 1
        for (int t = 0; t < K::TX; ++t) {
            const int task = threadIdx.x + t * K::THREADS;
            const unsigned off = 8u * (unsigned)((c * ROWS + task / N) * K::RS + phys<K>(task % N));
            float2 v[C];
#pragma unroll
            for (int k1 = 0; k1 < C; ++k1) v[k1] = dsmem_load(base[k1] + off);
            dft_reg<C, false>(v);
#pragma unroll
            for (int j1 = 0; j1 < C; ++j1) {
                const int i = (j1 ^ (C / 2)) * K::R + c * ROWS + task / N;
                if (i >= row_lo && i <= row_hi) dsmem_store(base[j1 ^ (C / 2)] + off, v[j1]);
            }
        }
    }
}

// P4 column transforms with two threads per column: lanes l and l ^ 16 of a
// warp share column position q; half h = lane / 16 holds local rows
// n2 and n2 + 16 for n2 in [8h, 8h + 8). The 32-point transform is split as
// 2 x 16: a radix-2 step with twiddles, an exchange of half the values with
// the partner lane, and a 16-point register DFT.
//
// Inverse: natural rows in, z[k] = X[h + 2k] out.
template <class K>
FPM_DEVICE void column_inverse_split(const float2* __restrict__ fld, int pq, int h, const float2* __restrict__ tw,
                                     float2 (&z)[16]) {
    float2 y0[8], y1[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const int n2 = 8 * h + i;
        const float2 a = fld[n2 * K::RS + pq], b = fld[(n2 + 16) * K::RS + pq];
        y0[i] = cadd(a, b);
        y1[i] = twiddle_smem<true>(csub(a, b), tw, 8 * n2);
    }
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const float2 send = h ? y0[i] : y1[i];
        const float2 recv = make_float2(__shfl_xor_sync(0xffffffffu, send.x, 16), __shfl_xor_sync(0xffffffffu, send.y, 16));
        const float2 own = h ? y1[i] : y0[i];
        z[i] = h ? recv : own;
        z[i + 8] = h ? own : recv;
    }
    dft_reg<16, true>(z);
}

// Forward, the dual: z[k] holds x'[h + 2k]; writes natural rows n2 and n2 + 16
// for n2 in [8h, 8h + 8), each times w_N^(-c * row) when the cluster splits
// the column (C > 1).
template <class K>
FPM_DEVICE void column_forward_split(float2* __restrict__ fld, int pq, int h, int c, const float2* __restrict__ tw,
                                     float2 (&z)[16]) {
    dft_reg<16, false>(z);
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const float2 send = h ? twiddle_smem<false>(z[i], tw, 8 * i) : z[i + 8];
        const float2 recv = make_float2(__shfl_xor_sync(0xffffffffu, send.x, 16), __shfl_xor_sync(0xffffffffu, send.y, 16));
        const float2 own = h ? twiddle_smem<false>(z[i + 8], tw, 8 * (i + 8)) : z[i];
        const float2 w0 = h ? recv : own, w1 = h ? own : recv;
        const int row = 8 * h + i;
        float2 lo = cadd(w0, w1), hi = csub(w0, w1);
        if constexpr (K::C > 1) {
            lo = twiddle_smem<false>(lo, tw, c * row * K::TW);
            hi = twiddle_smem<false>(hi, tw, c * (row + 16) * K::TW);
        }
        fld[row * K::RS + pq] = lo;
        fld[(row + 16) * K::RS + pq] = hi;
    }
}

// P4 column transforms for 16-row CTAs: one thread per column position,
// the 16 local rows in registers. Inverse: z[m] = sum_l X[l] w_16^{+lm}
// (spatial row c + C * m). Forward: the 16-point DFT, then the cluster
// twiddle w_N^(-c * b) on local row b ahead of the cross-CTA step.
template <class K>
FPM_DEVICE void column_inverse_local(const float2* __restrict__ fld, int pq, float2 (&z)[16]) {
#pragma unroll
    for (int l = 0; l < 16; ++l) z[l] = fld[l * K::RS + pq];
    dft_reg<16, true>(z);
}

template <class K>
FPM_DEVICE void column_forward_local(float2* __restrict__ fld, int pq, int c, const float2* __restrict__ tw,
                                     float2 (&z)[16]) {
    dft_reg<16, false>(z);
#pragma unroll
    for (int b = 0; b < 16; ++b) fld[b * K::RS + pq] = K::C > 1 ? twiddle_smem<false>(z[b], tw, c * b * K::TW) : z[b];
}

// End of a gradient-descent mini-batch (src/algorithms/gradient_descent.rs:
// 628-640): O -= (object_step / active) * G over the whole grid, then G = 0.
// The cluster's CTAs split the grid; one float4 holds two complex values.
template <class K>
FPM_DEVICE void gd_batch_apply(const TileDesc& T, float step, int c) {
    const long long total = (long long)T.M * (T.M + (T.M & 1)) / 2;
    const long long per = (total + K::C - 1) / K::C;
    const long long begin = c * per;
    const long long end = begin + per < total ? begin + per : total;
    float4* O4 = reinterpret_cast<float4*>(T.object);
    float4* G4 = reinterpret_cast<float4*>(T.gradient);
    float4* E4 = reinterpret_cast<float4*>(T.gradient_err);  // compensated: G's rounding error
    for (long long e = begin + threadIdx.x; e < end; e += K::THREADS) {
        float4 g = __ldcg(G4 + e);
        if (E4) {
            const float4 err = __ldcg(E4 + e);
            g.x -= err.x;
            g.y -= err.y;
            g.z -= err.z;
            g.w -= err.w;
            __stcg(E4 + e, make_float4(0.f, 0.f, 0.f, 0.f));
        }
        float4 o = __ldcg(O4 + e);
        o.x = fmaf(-step, g.x, o.x);
        o.y = fmaf(-step, g.y, o.y);
        o.z = fmaf(-step, g.z, o.z);
        o.w = fmaf(-step, g.w, o.w);
        __stcg(O4 + e, o);
        __stcg(G4 + e, make_float4(0.f, 0.f, 0.f, 0.f));
    }
}

// Pupil update of gradient descent at a batch end
// (src/algorithms/gradient_descent.rs:641-656, 688-690): this CTA's pupil
// rows move by -(pupil_step / active) * gradient, the accumulator is
// cleared, and the support is imposed. The caller's barriers order it.
template <class K>
FPM_DEVICE void gd_pupil_apply(const TileDesc& T, float2* __restrict__ pslab, const EngineParams& P, int c, float step) {
    const int i_lo = K::C == 1 ? 0 : c * K::R;
    __syncthreads();
    bool bad = false;
    for (int e = threadIdx.x; e < K::R * K::N; e += K::THREADS) {
        const size_t g = (size_t)i_lo * K::N + e;
        float2 p = cfma(-step, __ldcg(T.pupil_gradient + g), pslab[e]);
        bad |= !isfinite(p.x) || !isfinite(p.y);
        if (P.constrain_pupil && T.support[g] == 0) p = make_float2(0.f, 0.f);
        pslab[e] = p;
        __stcg(T.pupil_gradient + g, make_float2(0.f, 0.f));
    }
    if (bad) atomicOr(T.status, 64);
    __syncthreads();
}

template <class K>
FPM_DEVICE void load_pupil_slab(float2* __restrict__ pslab, const float2* __restrict__ pupil, int c) {
    for (int e = threadIdx.x; e < K::R * K::N; e += K::THREADS) {
        const int l = e / K::N, j = e % K::N;
        const int i = K::C == 1 ? l : c * K::R + l;
        pslab[e] = __ldcg(pupil + i * K::N + j);
    }
}

// The same rows as 16-byte asynchronous copies; the caller waits
// (cp.async.wait_all) and synchronises before the slab is read.
template <class K>
FPM_DEVICE void load_pupil_slab_async(float2* __restrict__ pslab, const float2* __restrict__ pupil, int c) {
    constexpr int PAIRS = K::N / 2;
    for (int e = threadIdx.x; e < K::R * PAIRS; e += K::THREADS) {
        const int l = e / PAIRS, j2 = e % PAIRS;
        const int i = K::C == 1 ? l : c * K::R + l;
        cp_async16(pslab + l * K::N + 2 * j2, pupil + (size_t)i * K::N + 2 * j2, 16);
    }
}

// Asynchronous copy of spectral step `step` into a shared descriptor slot
// (one 16-byte piece per thread of the first warp).
FPM_DEVICE void prefetch_step(SpectralStep* slot, const SpectralStep* steps, int step) {
    constexpr int PIECES = (int)(sizeof(SpectralStep) / 16);
    if (threadIdx.x < PIECES)
        cp_async16(reinterpret_cast<char*>(slot) + 16 * threadIdx.x,
                   reinterpret_cast<const char*>(steps + step) + 16 * threadIdx.x, 16);
}

// Sum of two FP64 values over every thread of the cluster, in a fixed order
// (warps, then CTAs by rank), identical in every CTA. `dred` holds a value
// per warp and `tred` this CTA's two totals; the closing barrier keeps them
// until every CTA has read them.
template <class K>
FPM_DEVICE void cluster_sum2(double& a, double& b, double* dred, double* tred) {
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    double part[2] = {a, b};
#pragma unroll
    for (int q = 0; q < 2; ++q) {
        const double w = warp_sum(part[q]);
        __syncthreads();
        if (lane == 0) dred[warp] = w;
        __syncthreads();
        if (tid == 0) {
            double t = 0.0;
            for (int ww = 0; ww < K::WARPS; ++ww) t += dred[ww];
            tred[q] = t;
        }
    }
    cluster_barrier<K>();
    if constexpr (K::C == 1) {
        a = tred[0];
        b = tred[1];
    } else {
        cg::cluster_group cluster = cg::this_cluster();
        a = b = 0.0;
        for (int r = 0; r < K::C; ++r) {
            const double* pr = cluster.map_shared_rank(tred, r);
            a += pr[0];
            b += pr[1];
        }
    }
    cluster_barrier<K>();
}

// One tile's whole launch (iterations [it_begin, it_end)) by one cluster.
template <int N_, int ALG, int LOSS>
FPM_DEVICE void engine_tile(const EngineParams& P, const int tile) {
    using K = Cfg<N_>;
    constexpr int N = K::N, R = K::R, C = K::C, NA = K::NA, NB = K::NB;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    float2* field = reinterpret_cast<float2*>(smem_raw);
    float2* fld = field + K::RS;  // FFT rows 0..31; raw row 0 is the U halo
    float2* osm = field + K::FIELD;
    float2* pslab = osm + K::STAGE;
    float2* tw = pslab + K::PSLAB;
    double* dred = reinterpret_cast<double*>(tw + 256);
    // TMA staging of the stencil: 256-point tiles of the fixed-pupil
    // families (the pupil-recovering ones are at their register limit),
    // whose staging slab starts 128-byte aligned.
    constexpr bool tma_capable = N_ == 256 && ALG != kAlgSpectral && ALG != kAlgEpry && ALG != kAlgEpryCal &&
                                 ALG != kAlgGlobalCal && ALG != kAlgGradientPupil &&
                                 (K::FIELD * 8) % 128 == 0;
    constexpr unsigned kStageBytes = (unsigned)(K::STAGE * sizeof(float2));
    __shared__ __align__(8) unsigned long long s_tma_bar;
    __shared__ int s_tma_failed;
    unsigned tma_phase = 0;
    double* tred = dred + K::WARPS;  // this CTA's truncation partials (residual, weight, |O|^2)
    float* fred = reinterpret_cast<float*>(dred + K::WARPS + 4);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int c = C == 1 ? 0 : (int)(blockIdx.x % C);
    // Tile and frame descriptors live in shared memory, not registers.
    __shared__ TileDesc s_tile;
    // Frame descriptor; spectral AP holds this step's descriptor and the
    // next one (prefetched) instead. Sized per family so the others keep
    // their shared-memory budget.
    __shared__ __align__(16) unsigned char s_desc[ALG == kAlgSpectral ? 2 * sizeof(SpectralStep) : sizeof(FrameParam)];
    FrameParam& s_frame = *reinterpret_cast<FrameParam*>(s_desc);
    // The next frame's descriptor, copied asynchronously one frame ahead.
    __shared__ __align__(16) FrameParam s_next;
    static_assert(sizeof(FrameParam) % 8 == 0, "FrameParam is copied in 8-byte pieces");
    int next_ready = -1;  // thread 0: order position whose descriptor s_next holds
    SpectralStep* const s_steps = reinterpret_cast<SpectralStep*>(s_desc);
    if (tid == 0) {
        s_tile = P.tiles[tile];
        if (tma_capable) {
            s_tma_failed = 0;
            mbar_init(&s_tma_bar, 1);
        }
    }
    for (int k = tid; k < 256; k += K::THREADS) tw[k] = c_tw256[k];
    __syncthreads();
    const TileDesc& T = s_tile;
    const bool use_tma = tma_capable && T.omap != nullptr && (smem_u32(osm) & 127u) == 0;
    const float eps = opaque((float)P.eps);  // epsilon in the per-pixel FP32 arithmetic
    const int M = T.M;
    const long long ostride = M + (M & 1);
    const int i_lo = C == 1 ? 0 : c * R;
    constexpr bool gradient = ALG == kAlgGradient || ALG == kAlgGradientTruncated || ALG == kAlgGradientPupil;
    constexpr bool projection = !gradient;
    // Families whose pupil evolves during the launch: per-frame maxima, all rows.
    constexpr bool gd_pupil = ALG == kAlgGradientPupil;
    constexpr bool epry = ALG == kAlgEpry || ALG == kAlgEpryCal;
    // EPRY with frame-gain / background recovery (either pupil mode).
    constexpr bool calibrating = ALG == kAlgEpryCal || ALG == kAlgGlobalCal;
    // Narrowband spectral AP: per-mode channel pupils and stored objects.
    constexpr bool spectral = ALG == kAlgSpectral;
    // Rows of psi that can be non-zero (all rows when the pupil evolves or
    // changes with the channel).
    const int row_lo = epry || gd_pupil || spectral ? 0 : T.row_lo;
    const int row_hi = epry || gd_pupil || spectral ? N - 1 : T.row_hi;

    load_pupil_slab<K>(pslab, T.pupil, c);
    int slab_channel = 0;  // spectral: channel whose pupil rows pslab holds
    int vstep = 0;         // spectral: steps taken in this launch (descriptor slot parity)
    if constexpr (spectral) {
        if (T.step_count > 0) prefetch_step(&s_steps[0], T.steps, 0);
    }
    int counter = P.momentum ? *T.counter : 0;
    double loss_acc = 0.0;
    // Mini-batch gradient descent: frames add into T.gradient and the object
    // moves once per batch of gd_batch consecutive frames of the order.
    const bool gd_batched = gradient && P.gd_batch > 1;
    int batch_active = 0;
    int pupil_active = 0;  // positive-weight frames since the last pupil update
    // Poisson truncation (src/algorithms/gradient_descent.rs:701-792): each
    // batch is walked twice, first forward-only for the residual statistic,
    // then with the gate |y - p| <= scale * sqrt(p) on the gradient.
    constexpr bool truncating = ALG == kAlgGradientTruncated;
    const int batch_len = gradient ? P.gd_batch : 1;
    double trunc_res = 0.0, trunc_pw = 0.0, trunc_norm = 0.0;
    float trunc_scale = 0.f;
    // Adaptive AP (src/algorithms/adaptive_alternating_projection.rs:245-307):
    // the per-tile step, identical in every CTA of the cluster.
    constexpr bool adaptive = ALG == kAlgLocalAdaptive;
    double ada_step = P.object_step;
    double ada_previous = 0.0;
    bool ada_has_previous = false;
    __syncthreads();

    for (int it = P.it_begin; it < P.it_end; ++it) {
        if (adaptive && it > P.it_begin) {
            // Objective of the pass just finished, from every CTA's partial.
            cluster_barrier<K>();
            double sum = 0.0;
            for (int r = 0; r < C; ++r) sum += __ldcg(T.partials + (size_t)(it - 1) * C + r);
            const double objective = T.weight_sum > 0.0 ? sum / T.weight_sum : NAN;
            if (!isfinite(objective) || objective < 0.0) {
                if (tid == 0) atomicOr(T.status, 32);
            } else {
                if (ada_has_previous) {
                    const double progress = (ada_previous - objective) / fmax(ada_previous, (double)P.eps);
                    if (progress <= P.progress_threshold)
                        ada_step = fmax(ada_step * P.reduction_factor, P.minimum_step);
                }
                ada_previous = objective;
                ada_has_previous = true;
            }
        }
        const int steps = truncating ? 2 * T.frame_count : spectral ? T.step_count : T.frame_count;
        const int step_begin = P.frame_end > 0 ? P.frame_begin : 0;
        const int step_end = P.frame_end > 0 ? min(P.frame_end, steps) : steps;
        for (int step = step_begin; step < step_end; ++step) {
            // Truncating: batch k covers steps [2kB, 2kB + 2b): b statistics
            // steps, then the b update steps of the same frames.
            int idx = step;
            bool stats = false;
            if (truncating) {
                const int k = step / (2 * batch_len), base = k * batch_len;
                const int blen = min(batch_len, T.frame_count - base), within = step - 2 * k * batch_len;
                stats = within < blen;
                idx = base + (stats ? within : within - blen);
                if (within == 0) {
                    // Batch start: |O|^2 of this CTA's share of the grid.
                    const long long total = (long long)M * ostride;
                    const long long per = (total + C - 1) / C;
                    const long long begin = c * per;
                    const long long end = begin + per < total ? begin + per : total;
                    double nacc = 0.0;
                    for (long long e = begin + tid; e < end; e += K::THREADS) {
                        if ((int)(e % ostride) >= M) continue;  // padding column
                        const float2 o = __ldcg(T.object + e);
                        nacc += (double)o.x * o.x + (double)o.y * o.y;
                    }
                    trunc_norm = nacc;
                    trunc_res = trunc_pw = 0.0;
                }
                if (within == blen) {
                    // First update step: reduce the statistic over the cluster
                    // in a fixed order, identically in every CTA.
                    const double part[3] = {trunc_res, trunc_pw, trunc_norm};
#pragma unroll
                    for (int q = 0; q < 3; ++q) {
                        const double w = warp_sum(part[q]);
                        __syncthreads();
                        if (lane == 0) dred[warp] = w;
                        __syncthreads();
                        if (tid == 0) {
                            double t = 0.0;
                            for (int ww = 0; ww < K::WARPS; ++ww) t += dred[ww];
                            tred[q] = t;
                        }
                    }
                    cluster_barrier<K>();
                    double tot[3] = {0.0, 0.0, 0.0};
                    if constexpr (C == 1) {
                        tot[0] = tred[0];
                        tot[1] = tred[1];
                        tot[2] = tred[2];
                    } else {
                        cg::cluster_group cluster = cg::this_cluster();
                        for (int r = 0; r < C; ++r) {
                            const double* pr = cluster.map_shared_rank(tred, r);
                            tot[0] += pr[0];
                            tot[1] += pr[1];
                            tot[2] += pr[2];
                        }
                    }
                    const double rms = fmax(sqrt(tot[2]), sqrt((double)P.eps));
                    const double mean = tot[1] > 0.0 ? tot[0] / tot[1] : 0.0;
                    const double sc = (double)P.trunc_threshold * mean / rms;
                    trunc_scale = (float)sc;
                    if (!isfinite(sc) || sc < 0.0) {
                        trunc_scale = 0.f;
                        if (tid == 0) atomicOr(T.status, 16);
                    }
                    cluster_barrier<K>();  // partials read before the next batch rewrites them
                }
            }
            if constexpr (spectral) {
                // This step's descriptor arrived during the previous step; the
                // slot of the previous step is free again (its readers passed
                // that step's closing barrier) and takes the next descriptor.
                cp_async_wait_all();
                __syncthreads();
                const int next = step + 1 < steps ? step + 1 : 0;
                prefetch_step(&s_steps[(vstep + 1) & 1], T.steps, next);
            } else {
                const int f0 = T.order ? __ldg(T.order + idx) : idx;
                if (tid == 0) {
                    if (next_ready == idx) {
                        cp_async_wait_all();
                        s_frame = s_next;
                    } else {
                        s_frame = T.params[f0];
                    }
                    // The next frame's descriptor comes in behind this frame,
                    // and its measurement rows of this CTA go to L2 now, so
                    // that its P4 loads do not wait on HBM.
                    if (!truncating && idx + 1 < step_end) {
                        const int f1 = T.order ? __ldg(T.order + idx + 1) : idx + 1;
#pragma unroll
                        for (int k = 0; k < (int)(sizeof(FrameParam) / 8); ++k)
                            cp_async8(reinterpret_cast<char*>(&s_next) + 8 * k,
                                      reinterpret_cast<const char*>(T.params + f1) + 8 * k);
                        next_ready = idx + 1;
                        const size_t off = (size_t)f1 * N * N + (size_t)c * R * N;
                        prefetch_l2(T.meas + off, R * N * sizeof(float));
                        if (T.masks) prefetch_l2(T.masks + off, R * N);
                    }
                }
                __syncthreads();
            }
            const SpectralStep& sp = s_steps[vstep & 1];
            ++vstep;
            const int f = spectral ? sp.exposure : T.order ? T.order[idx] : idx;
            const FrameParam& fp = spectral ? sp.frame : s_frame;
            // Spectral update steps start from the stored mode field: no
            // inverse transform; the object stencil for P8 and a changed
            // channel's pupil rows arrive asynchronously behind P4-P6.
            const bool spectral_update = spectral && sp.update == 1;  // update only: no staging or inverse
            float2* const obj = spectral ? T.object + (size_t)sp.object * M * ostride : T.object;
            if constexpr (spectral) {
                if (sp.channel != slab_channel) {
                    // Previous readers of pslab finished behind the last step's barriers.
                    load_pupil_slab_async<K>(pslab, T.pupil + (size_t)sp.channel * N * N, c);
                    slab_channel = sp.channel;
                }
                if (spectral_update) stage_object<K, false>(osm, obj, M, ostride, fp, i_lo, row_lo, row_hi);
            }
            const bool batch_boundary = gradient && !stats && ((idx + 1) % P.gd_batch == 0 || idx + 1 == T.frame_count);
            const bool batch_end = gd_batched && batch_boundary;
            if (fp.weight == 0.0f) {
                __syncthreads();
                if constexpr (gd_pupil) {
                    if (batch_boundary) {
                        if (pupil_active > 0) gd_pupil_apply<K>(T, pslab, P, c, (float)(P.pupil_step / pupil_active));
                        pupil_active = 0;
                    }
                }
                if (batch_end) {
                    if (batch_active > 0) gd_batch_apply<K>(T, (float)(P.object_step / batch_active), c);
                    batch_active = 0;
                    cluster_barrier<K>();
                }
                continue;
            }
            if (gd_batched && !stats) ++batch_active;
            if (gd_pupil && !stats) ++pupil_active;

            // S0
            if (use_tma && !s_tma_failed) {
                // One bulk tensor load of the (R + 1) x (N + 2) stencil from an
                // even column (pair c0 / 2); rows and pairs past the grid read
                // as zeros. CTAs the pupil leaves empty stage nothing.
                const int r_begin = max(row_lo - i_lo, 0), r_end = min(row_hi + 1 - i_lo, R);
                if (r_begin <= r_end) {
                    if (tid == 0) {
                        mbar_arrive_expect_tx(&s_tma_bar, kStageBytes);
                        tma_load_3d(osm, T.omap, 0, (fp.lower_col & ~1) >> 1, fp.lower_row + i_lo, &s_tma_bar);
                    }
                    if (!mbar_wait(&s_tma_bar, tma_phase)) {
                        s_tma_failed = 1;
                        atomicOr(T.status, 512);
                    }
                    tma_phase ^= 1u;
                }
            } else if (!spectral_update) {
                stage_object<K>(osm, obj, M, ostride, fp, i_lo, row_lo, row_hi);
            }
            if (!spectral) __syncthreads();
            if (spectral && !spectral_update) __syncthreads();
            const float2* ostage = osm + (fp.lower_col & 1);

            // P1, P2
            float max_obj = 0.f, max_pup = 0.f;
            if (!spectral_update)
                rows_inverse<K, epry || gd_pupil>(fld, ostage, tw, pslab, fp, c, i_lo, row_lo, row_hi, max_obj,
                                                  max_pup);
            if constexpr (epry || gd_pupil) {
                max_obj = warp_max(max_obj);
                max_pup = warp_max(max_pup);
                if (lane == 0) {
                    fred[warp] = max_obj;
                    fred[K::WARPS + warp] = max_pup;
                }
                __syncthreads();
                if (tid == 0) {
                    float a = 0.f, b = 0.f;
                    for (int w = 0; w < K::WARPS; ++w) {
                        a = fmaxf(a, fred[w]);
                        b = fmaxf(b, fred[K::WARPS + w]);
                    }
                    fred[2 * K::WARPS] = a;
                    fred[2 * K::WARPS + 1] = b;
                }
            }
            if (!spectral_update) cluster_barrier<K>();

            float frame_max_obj = 0.f, frame_max_pup = 0.f;
            if constexpr (epry || gd_pupil) {
                if constexpr (C == 1) {
                    frame_max_obj = fred[2 * K::WARPS];
                    frame_max_pup = fred[2 * K::WARPS + 1];
                } else {
                    cg::cluster_group cluster = cg::this_cluster();
#pragma unroll
                    for (int r = 0; r < C; ++r) {
                        const float* pf = cluster.map_shared_rank(fred, r);
                        frame_max_obj = fmaxf(frame_max_obj, pf[2 * K::WARPS]);
                        frame_max_pup = fmaxf(frame_max_pup, pf[2 * K::WARPS + 1]);
                    }
                }
            }

            // P3
            if constexpr (C > 1) {
                if (!spectral_update) columns_cross_inverse<K>(fld, tw, c, row_lo, row_hi);
            }
            // P4 ownership. R = 32: column position q4, half h4, slot k =
            // local spatial row h4 + 2k. R = 16: column position tid, slot k =
            // local row k. Local row m of CTA c is spatial row c + C * m, and
            // the engine layout stores it at (c * R + m) * N + q.
            const int q4 = R == 32 ? (warp << 4) | (lane & 15) : tid, h4 = R == 32 ? lane >> 4 : 0;
            const int mbase = (c * R + h4) * N + q4;
            constexpr int mstride = R == 32 ? 2 * N : N;

            if constexpr (C > 1) {
                if (!spectral_update) cluster_barrier<K>();
            }

            if constexpr (spectral) {
                // P4 of spectral AP (src/algorithms/spectral.rs:218-270). Each
                // thread owns the same detector pixels in every step, so the
                // mode fields and the prediction need no synchronisation.
                float2 v[16];
                float2* const slot = T.mode_fields + (size_t)sp.slot * N * N + mbase;
                float* const pred = T.prediction + mbase;
                const int pq = phys<K>(q4);
                // The exposure's last mode evaluates and updates in one step
                // (kind 2): the prediction is then complete and the staged
                // stencil is still the current object. Its psi goes through
                // the scratch like the others (registers are the limit).
                const bool merged = sp.update == 2;
                if (!spectral_update) {
                    // Evaluation: psi_k, and prediction += w_k |psi_k|^2.
                    if constexpr (R == 32) column_inverse_split<K>(fld, pq, h4, tw, v);
                    else column_inverse_local<K>(fld, pq, v);
#pragma unroll
                    for (int k = 0; k < 16; ++k) {
                        __stcg(slot + (size_t)k * mstride, v[k]);
                        float pk = sp.mode_weight * cnorm2(v[k]);
                        if (sp.slot > 0) pk += __ldcg(pred + (size_t)k * mstride);
                        __stcg(pred + (size_t)k * mstride, pk);
                    }
                    if (!merged) {
                        __syncthreads();
                        continue;
                    }
                }
                // Update: psi' - psi with the exposure's shared amplitude
                // ratio sqrt(target / prediction); masked pixels keep psi and
                // dark pixels take sqrt(target / weight sum).
                const size_t off = (size_t)f * N * N + mbase;
                const float gain = sp.gain, inv_gain = 1.0f / sp.gain, bg = sp.background;
                const bool first = sp.first_update != 0;
                float frame_loss = 0.f;
#pragma unroll
                for (int k = 0; k < 16; ++k) {
                    const float meas = __ldcs(T.meas + off + (size_t)k * mstride);
                    const bool masked = T.masks && T.masks[off + (size_t)k * mstride] == 0;
                    const float2 psi = __ldcg(slot + (size_t)k * mstride);
                    const float pk = __ldcg(pred + (size_t)k * mstride);
                    if (masked) {
                        v[k] = make_float2(0.f, 0.f);
                        continue;
                    }
                    if (first) frame_loss += point_loss<LOSS>(fmaf(gain, pk, bg), meas, P.loss);
                    const float target = fmaxf((meas - bg) * inv_gain, 0.f);
                    if (pk > eps)
                        v[k] = cscale(psi, sqrtf(target / pk) - 1.f);
                    else
                        v[k] = make_float2(sqrtf(target * sp.inv_weight_sum) - psi.x, -psi.y);
                }
                if constexpr (R == 32) column_forward_split<K>(fld, pq, h4, c, tw, v);
                else column_forward_local<K>(fld, pq, c, tw, v);
                if (first) loss_acc += (double)frame_loss * sp.loss_scale;
            } else {
            // P4: column inverse FFT, projection, column forward FFT.
            {
                const float* brow =
                    T.background ? T.background + (size_t)f * T.background_stride + mbase : nullptr;
                float gain = fp.gain, inv_gain = 1.0f / fp.gain;
                const int pq = phys<K>(q4);
                float2 v[16];
                if constexpr (R == 32) column_inverse_split<K>(fld, pq, h4, tw, v);
                else column_inverse_local<K>(fld, pq, v);
                // Measurements are loaded next to their use: a prefetch ahead
                // of the cluster barrier measured slower.
                float mreg[16];
                unsigned mbits = 0xffffu;
                {
                    const size_t off = (size_t)f * N * N + mbase;
#pragma unroll
                    for (int k = 0; k < 16; ++k) mreg[k] = __ldcs(T.meas + off + (size_t)k * mstride);
                    if (T.masks) {
                        mbits = 0u;
#pragma unroll
                        for (int k = 0; k < 16; ++k) mbits |= (T.masks[off + (size_t)k * mstride] != 0 ? 1u : 0u) << k;
                    }
                }
                // EPRY frame-gain and background recovery (update_gain and
                // update_background, src/algorithms/common.rs:390-489): the
                // frame's gain moves toward sum p (y - b)+ / sum p^2 and its
                // background by the mean residual y - g p - b, from the
                // prediction p = |psi|^2 before the projection; both are
                // summed over the cluster in FP64 and the projection below
                // uses the new values. The amplitude form holds
                // a = sqrt(max(y / g0, 0)); its intensities are g0 a^2.
                bool recovered = false;
                float bgv[16];
                if constexpr (calibrating) {
                    {
                        recovered = true;
                        if (T.amplitude) {
                            mbits = 0u;
#pragma unroll
                            for (int k = 0; k < 16; ++k) {
                                const float a = mreg[k];
                                if (a >= 0.f) mbits |= 1u << k;
                                mreg[k] = a >= 0.f ? fp.gain * (a * a) : 0.f;
                            }
                        }
                        const TileRecovery rs = P.recovery[tile];
                        float* const bstate = rs.bg_state ? rs.bg_state + (size_t)f * N * N + mbase : nullptr;
#pragma unroll
                        for (int k = 0; k < 16; ++k) bgv[k] = bstate ? bstate[k * mstride] : 0.f;
                        double g = rs.gain_state[f];
                        if (P.recover_gains) {
                            double num = 0.0, den = 0.0;
#pragma unroll
                            for (int k = 0; k < 16; ++k) {
                                if (((mbits >> k) & 1u) == 0u) continue;
                                const double pk = (double)cnorm2(v[k]);
                                num += pk * fmax((double)mreg[k] - (double)bgv[k], 0.0);
                                den += pk * pk;
                            }
                            cluster_sum2<K>(num, den, dred, tred);
                            if (den > P.eps) {
                                const double est = fmin(fmax(num / den, P.gain_min), P.gain_max);
                                g = fmin(fmax((1.0 - P.gain_step) * g + P.gain_step * est, P.gain_min), P.gain_max);
                                if (c == 0 && tid == 0) rs.gain_state[f] = g;
                            }
                        }
                        if (P.recover_background) {
                            double res = 0.0, cnt = 0.0;
#pragma unroll
                            for (int k = 0; k < 16; ++k) {
                                if (((mbits >> k) & 1u) == 0u) continue;
                                res += (double)mreg[k] - g * (double)cnorm2(v[k]) - (double)bgv[k];
                                cnt += 1.0;
                            }
                            cluster_sum2<K>(res, cnt, dred, tred);
                            if (cnt > 0.0) {
                                const double corr = P.background_step * res / cnt;
#pragma unroll
                                for (int k = 0; k < 16; ++k) {
                                    bgv[k] = (float)fmin(fmax((double)bgv[k] + corr, P.background_min), P.background_max);
                                    bstate[k * mstride] = bgv[k];
                                }
                            }
                        }
                        gain = (float)g;
                        inv_gain = 1.0f / gain;
                    }
                }
                if constexpr (truncating) {
                    if (stats) {
                        // Statistic: |y - p| and the count over unmasked pixels.
                        float res = 0.f, cnt = 0.f;
#pragma unroll
                        for (int k = 0; k < 16; ++k) {
                            const float intrinsic = cnorm2(v[k]);
                            float target;
                            bool valid;
                            if (T.amplitude) {
                                valid = mreg[k] >= 0.f;
                                target = mreg[k] * mreg[k];
                            } else {
                                valid = ((mbits >> k) & 1u) != 0u;
                                const float bg = brow ? __ldg(brow + k * mstride) : 0.f;
                                target = fmaxf((mreg[k] - bg) * inv_gain, 0.f);
                            }
                            if (valid) {
                                res += fabsf(target - intrinsic);
                                cnt += 1.f;
                            }
                        }
                        trunc_res += (double)fp.weight * res;
                        trunc_pw += (double)fp.weight * cnt;
                    }
                }
                float frame_loss = 0.f;
                if (stats) {
                    // Forward-only statistics step: nothing to write back.
                } else if (T.amplitude && !recovered) {
                    // a = sqrt(max(I / g, 0)), -1 where masked; with no
                    // background, I = g a^2 exactly as the reference uses it.
#pragma unroll
                    for (int k = 0; k < 16; ++k) {
                        const float a = mreg[k];
                        const float intrinsic = cnorm2(v[k]);
                        const float r = rsqrtf(fmaxf(intrinsic, 1.17549435e-38f));
                        const float s_amp = intrinsic * r;
                        if constexpr (projection) {
                            // The forward transform takes psi' - psi, so P7 reads
                            // Psi' - P * patch directly; masked pixels keep psi.
                            if (a >= 0.f) {
                                if constexpr (LOSS == 0) {
                                    const float d = s_amp - a;
                                    frame_loss = fmaf(d, d, frame_loss);
                                } else {
                                    frame_loss += point_loss<LOSS>(gain * intrinsic, gain * a * a, P.loss);
                                }
                                v[k] = intrinsic > eps ? cscale(v[k], fmaf(a, r, -1.f))
                                                         : make_float2(a - v[k].x, -v[k].y);
                            } else {
                                v[k] = make_float2(0.f, 0.f);
                            }
                        } else {
                            if (a < 0.f) {
                                v[k] = make_float2(0.f, 0.f);
                            } else if constexpr (LOSS == 0) {
                                const float d = s_amp - a;
                                frame_loss = fmaf(d, d, frame_loss);
                                v[k] = cscale(v[k], 1.f - a * rsqrtf(fmaxf(intrinsic, eps)));
                            } else {
                                const float target = a * a;
                                frame_loss += point_loss<LOSS>(intrinsic, target, P.loss);
                                const bool kept = !truncating || fabsf(target - intrinsic) <= trunc_scale * sqrtf(intrinsic);
                                v[k] = cscale(v[k], kept ? descent_factor<LOSS>(intrinsic, target, P.loss, eps) : 0.f);
                            }
                        }
                    }
                    // Amplitude MSE of the projection family is gain * (sqrt(intrinsic) - a)^2.
                    if (projection && LOSS == 0) frame_loss *= gain;
                } else {
#pragma unroll
                    for (int k = 0; k < 16; ++k) {
                        const float meas = mreg[k];
                    const bool masked = ((mbits >> k) & 1u) == 0u;
                    const float bg = recovered ? bgv[k] : brow ? __ldg(brow + k * mstride) : 0.f;
                    const float intrinsic = cnorm2(v[k]);
                    const float target = fmaxf((meas - bg) * inv_gain, 0.f);
                    if constexpr (projection) {
                        if (!masked) {
                            frame_loss += point_loss<LOSS>(fmaf(gain, intrinsic, bg), meas, P.loss);
                            v[k] = intrinsic > eps ? cscale(v[k], fmaf(sqrtf(target), rsqrtf(intrinsic), -1.f))
                                                     : make_float2(sqrtf(target) - v[k].x, -v[k].y);
                        } else {
                            v[k] = make_float2(0.f, 0.f);
                        }
                    } else {
                        if (masked) {
                            v[k] = make_float2(0.f, 0.f);
                        } else {
                            frame_loss += point_loss<LOSS>(intrinsic, target, P.loss);
                            const bool kept = !truncating || fabsf(target - intrinsic) <= trunc_scale * sqrtf(intrinsic);
                            v[k] = cscale(v[k], kept ? descent_factor<LOSS>(intrinsic, target, P.loss, eps) : 0.f);
                        }
                    }
                    }
                }
                if (!stats) {
                    if constexpr (R == 32) column_forward_split<K>(fld, pq, h4, c, tw, v);
                    else column_forward_local<K>(fld, pq, c, tw, v);
                    loss_acc += (double)frame_loss * fp.loss_scale;
                }
            }
            }  // non-spectral P4
            if (stats) {
                __syncthreads();
                continue;
            }
            cluster_barrier<K>();

            // P5
            if constexpr (C > 1) {
                columns_cross_forward<K>(fld, c, row_lo, row_hi);
                cluster_barrier<K>();
            }

            // P6: row FFT step C' with twiddles.
#pragma unroll 1
            for (int t = 0; t < K::T2; ++t) {
                const int task = tid + t * K::THREADS;
                const int l = task / NA, ka = task % NA;
                const int i = centred_row<K>(c, l);
                if (i < row_lo || i > row_hi) continue;
                float2* g = fld + l * K::RS + ka * (NB + 1);
                float2 v[NB];
#pragma unroll
                for (int kb = 0; kb < NB; ++kb) v[kb] = g[kb];
                dft_reg<NB, false>(v);
#pragma unroll
                for (int jb = 0; jb < NB; ++jb) g[jb] = twiddle_smem<false>(v[jb], tw, ka * jb * K::TW);
            }
            // Spectral update steps: the pupil rows and object stencil copied
            // since the step start are needed from P7 on.
            if (spectral_update) cp_async_wait_all();
            __syncthreads();

            // P7: row FFT step A', fftshift, correction U (+ EPRY pupil update).
            // P4 transformed psi' - psi, so psi below is already Psi' - P * patch
            // (src/algorithms/common.rs:186-196); the patch itself is needed only
            // by the pupil updates.
            {
                const float inv_n2 = 1.0f / (float)(N * N);
                // The frame's scalars in FP64, each rounded once.
                const double max_p2 =
                    epry || gd_pupil ? (double)fmaxf(frame_max_pup, eps) : T.max_pupil_power;
                const double obj_den = (double)fmaxf(frame_max_obj, eps) + P.eps;
                // Pupil gradient weight w * (N^2 / valid) / (max |patch|^2 + eps).
                const float pupil_grad_scale =
                    opaque(gd_pupil ? (float)((double)fp.weight * fp.valid_scale / obj_den) : 0.f);
                const float inv_global = opaque((float)(1.0 / (max_p2 + P.eps)));
                const float pupil_scale = opaque(epry ? (float)((double)fp.weight * P.pupil_step / obj_den) : 0.f);
                // rPIE: 1 / ((1 - alpha) |P|^2 + alpha max|P|^2 + eps) = 1 / (rpie_a |P|^2 + rpie_b).
                const float rpie_a = opaque((float)(1.0 - P.alpha)), rpie_b = opaque((float)(P.alpha * max_p2 + P.eps));
                // U of one task (row l, column class jb) into v, from the row's
                // transform in v: pixels j = (NB * ja + jb + N / 2) mod N.
                auto correction = [&](float2 (&v)[NA], int i, int jb) {
                    const int il = i - i_lo;
#pragma unroll
                    for (int ja = 0; ja < NA; ++ja) {
                        const int j = (NB * ja + jb + N / 2) & (N - 1);
                        const float2 psi = cscale(v[ja], inv_n2);
                        float2* pp = pslab + il * N + j;
                        const float2 pv = *pp;
                        float2 u;
                        if constexpr (projection) {
                            const float pw = cnorm2(pv);
                            float inv_den;
                            if constexpr (ALG == kAlgLocal || ALG == kAlgLocalAdaptive || spectral)
                                inv_den = 1.0f / (pw + eps);
                            else if constexpr (ALG == kAlgRpie)
                                inv_den = 1.0f / fmaf(rpie_a, pw, rpie_b);
                            else
                                inv_den = inv_global;
                            u = cscale(cmulc(psi, pv), inv_den);
                            if constexpr (epry) {
                                const float2 pt = patch_at(ostage, K::ORS, il, j, fp);
                                float2 np = cfma(pupil_scale, cmulc(psi, pt), pv);
                                if (P.constrain_pupil && T.support[i * N + j] == 0) np = make_float2(0.f, 0.f);
                                *pp = np;
                            }
                        } else {
                            u = cscale(cmulc(psi, pv), inv_global);
                            if constexpr (gd_pupil) {
                                const float2 pt = patch_at(ostage, K::ORS, il, j, fp);
                                float2* g = T.pupil_gradient + (size_t)i * N + j;
                                __stcg(g, cfma(pupil_grad_scale, cmulc(psi, pt), __ldcg(g)));
                            }
                        }
                        v[ja] = u;
                    }
                };
                if constexpr (C > 1) {
                    // Each row's NB tasks sit in one warp (32 % NB == 0) and
                    // centred row i is local row l, so U overwrites the row
                    // in place once the warp has read it.
                    static_assert(32 % NB == 0, "a warp holds whole rows");
                    float2* next_halo = c < C - 1 ? cg::this_cluster().map_shared_rank(field, c + 1) : nullptr;
#pragma unroll 1
                    for (int t = 0; t < K::T1; ++t) {
                        const int task = tid + t * K::THREADS;
                        const int l = task / NB, jb = task % NB;
                        const int i = centred_row<K>(c, l);
                        const bool live = i >= row_lo && i <= row_hi;
                        float2 v[NA];
#pragma unroll
                        for (int ka = 0; ka < NA; ++ka)
                            v[ka] = live ? fld[l * K::RS + phys<K>(NB * ka + jb)] : make_float2(0.f, 0.f);
                        __syncwarp();
                        if (live) {
                            dft_reg<NA, false>(v);
                            correction(v, i, jb);
                        }
#pragma unroll
                        for (int ja = 0; ja < NA; ++ja) {
                            const int j = (NB * ja + jb + N / 2) & (N - 1);
                            fld[l * K::RS + j] = v[ja];
                            if (l == R - 1 && next_halo) next_halo[j] = v[ja];
                        }
                    }
                } else {
                    // One CTA: fftshift moves U to the row N / 2 away, which
                    // another warp reads, so U waits in registers.
                    float2 ureg[K::T1][NA];
#pragma unroll
                    for (int t = 0; t < K::T1; ++t) {
                        const int task = tid + t * K::THREADS;
                        const int l = task / NB, jb = task % NB;
                        const int i = centred_row<K>(c, l);
                        if (i < row_lo || i > row_hi) {
#pragma unroll
                            for (int ja = 0; ja < NA; ++ja) ureg[t][ja] = make_float2(0.f, 0.f);
                            continue;
                        }
#pragma unroll
                        for (int ka = 0; ka < NA; ++ka) ureg[t][ka] = fld[l * K::RS + phys<K>(NB * ka + jb)];
                        dft_reg<NA, false>(ureg[t]);
                        correction(ureg[t], i, jb);
                    }
                    __syncthreads();
#pragma unroll
                    for (int t = 0; t < K::T1; ++t) {
                        const int task = tid + t * K::THREADS;
                        const int l = task / NB, jb = task % NB;
                        const int urow = centred_row<K>(c, l) - i_lo;
#pragma unroll
                        for (int ja = 0; ja < NA; ++ja) {
                            const int j = (NB * ja + jb + N / 2) & (N - 1);
                            fld[urow * K::RS + j] = ureg[t][ja];
                        }
                    }
                }
            }
            cluster_barrier<K>();

            // P8: exact bilinear adjoint scatter of scale * U into the object.
            {
                // Projection: O += w * step * adj(U). Gradient descent: O -= step *
                // w * (N^2 / valid) * adj(U), or with mini-batches G += w *
                // (N^2 / valid) * adj(U).
                const float scale = opaque(spectral     ? (float)((double)sp.update_scale * P.object_step)
                                           : projection ? (float)((double)fp.weight * (adaptive ? ada_step : P.object_step))
                                           : gd_batched ? fp.weight * fp.valid_scale
                                                        : (float)(-P.object_step * (double)fp.weight * fp.valid_scale));
                // Spectral updates stage the current object at the step start: an
                // earlier mode of the same exposure may have changed it.
                float2* target = gd_batched ? T.gradient : obj;
                float2* const comp_err = spectral ? nullptr : gd_batched ? T.gradient_err : T.object_err;
                const int rows8 = C == 1 ? N + fp.has_upper_row : R + (c == C - 1 ? fp.has_upper_row : 0);
                const int cols8 = N + fp.has_upper_col;
                constexpr int PER = (N + 1 + 31) / 32;
                for (int r = warp; r < rows8; r += K::WARPS) {
                    const int i = i_lo + r;
                    // Object row i takes U rows i and i - 1: both zero outside [row_lo, row_hi + 1].
                    if (i < row_lo || i > row_hi + 1) continue;
                    const bool has0 = i < N, has1 = i >= 1;
                    const float2* u0 = fld + r * K::RS;
                    const float2* u1 = u0 - K::RS;  // r == 0: the halo row
                    const float2* srow = ostage + r * K::ORS;
                    float2* grow = target + (long long)(fp.lower_row + i) * ostride + fp.lower_col;
                    // The bilinear adjoint of U at stencil column j.
                    auto adjoint = [&](int j) {
                        const float2 z = make_float2(0.f, 0.f);
                        const float2 a = has0 && j < N ? u0[j] : z;
                        const float2 b = has0 && j >= 1 && j <= N ? u0[j - 1] : z;
                        const float2 d0 = has1 && j < N ? u1[j] : z;
                        const float2 d1 = has1 && j >= 1 && j <= N ? u1[j - 1] : z;
                        float2 acc = cscale(a, fp.w00);
                        acc = cfma(fp.w01, b, acc);
                        acc = cfma(fp.w10, d0, acc);
                        return cfma(fp.w11, d1, acc);
                    };
                    if (comp_err) {
                        // Kahan: add scale * acc minus the carried error and keep
                        // the new error (what the rounded sum lost), cell by cell.
                        float2* erow = comp_err + (grow - target);
#pragma unroll 1
                        for (int j = lane; j < cols8; j += 32) {
                            const float2 acc = adjoint(j);
                            const float2 base = gd_batched ? __ldcg(grow + j) : srow[j];
                            const float2 e = __ldcg(erow + j);
                            const float2 y = make_float2(fmaf(scale, acc.x, -e.x), fmaf(scale, acc.y, -e.y));
                            const float2 sum = cadd(base, y);
                            __stcg(grow + j, sum);
                            __stcg(erow + j, make_float2((sum.x - base.x) - y.x, (sum.y - base.y) - y.y));
                        }
                        continue;
                    }
                    float2 out[PER];
#pragma unroll
                    for (int t = 0; t < PER; ++t) {
                        const int j = lane + 32 * t;
                        const float2 z = make_float2(0.f, 0.f);
                        const float2 acc = adjoint(j);
                        const float2 base = j < cols8 ? (gd_batched ? __ldcg(grow + j) : srow[j]) : z;
                        out[t] = j < cols8 ? cfma(scale, acc, base) : z;
                    }
#pragma unroll
                    for (int t = 0; t < PER; ++t) {
                        const int j = lane + 32 * t;
                        if (j < cols8) __stcg(grow + j, out[t]);
                    }
                }
            }
            cluster_barrier<K>();

            if constexpr (gd_pupil) {
                if (batch_boundary) {
                    gd_pupil_apply<K>(T, pslab, P, c, (float)(P.pupil_step / pupil_active));
                    pupil_active = 0;
                }
            }
            if (batch_end) {
                gd_batch_apply<K>(T, (float)(P.object_step / batch_active), c);
                batch_active = 0;
                cluster_barrier<K>();
            }

            // mPIE momentum event (src/algorithms/common.rs:308-387).
            if (P.momentum) {
                counter += 1;
                if (counter >= P.interval) {
                    counter = 0;
                    const long long total = (long long)M * ostride / 2;  // float4 = two complex values
                    const long long per = (total + C - 1) / C;
                    const long long begin = c * per;
                    const long long end = begin + per < total ? begin + per : total;
                    float4* O4 = reinterpret_cast<float4*>(T.object);
                    float4* V4 = reinterpret_cast<float4*>(T.velocity);
                    float4* A4 = reinterpret_cast<float4*>(T.anchor);
                    bool bad = false;
                    constexpr int U = 4;
                    for (long long e0 = begin + tid; e0 < end; e0 += (long long)K::THREADS * U) {
                        float4 o[U], v[U], a[U];
#pragma unroll
                        for (int u = 0; u < U; ++u) {
                            const long long e = e0 + (long long)u * K::THREADS;
                            if (e < end) {
                                o[u] = __ldcg(O4 + e);
                                v[u] = __ldcg(V4 + e);
                                a[u] = __ldcg(A4 + e);
                            }
                        }
#pragma unroll
                        for (int u = 0; u < U; ++u) {
                            const long long e = e0 + (long long)u * K::THREADS;
                            if (e < end) {
                                float4 nv, no;
                                nv.x = fmaf(P.friction, v[u].x, o[u].x - a[u].x);
                                nv.y = fmaf(P.friction, v[u].y, o[u].y - a[u].y);
                                nv.z = fmaf(P.friction, v[u].z, o[u].z - a[u].z);
                                nv.w = fmaf(P.friction, v[u].w, o[u].w - a[u].w);
                                if (P.feedback == 0.f) {
                                    no = o[u];
                                } else {
                                    no.x = fmaf(P.feedback, nv.x, o[u].x);
                                    no.y = fmaf(P.feedback, nv.y, o[u].y);
                                    no.z = fmaf(P.feedback, nv.z, o[u].z);
                                    no.w = fmaf(P.feedback, nv.w, o[u].w);
                                }
                                bad |= !isfinite(nv.x) || !isfinite(nv.y) || !isfinite(nv.z) || !isfinite(nv.w) ||
                                       !isfinite(no.x) || !isfinite(no.y) || !isfinite(no.z) || !isfinite(no.w);
                                __stcg(V4 + e, nv);
                                __stcg(O4 + e, no);
                                __stcg(A4 + e, no);
                            }
                        }
                    }
                    if (bad) atomicOr(T.status, 1);
                    cluster_barrier<K>();
                }
            }
        }
        // Objective partial for this iteration and CTA (deterministic order).
        double s = warp_sum(loss_acc);
        loss_acc = 0.0;
        if (lane == 0) dred[warp] = s;
        __syncthreads();
        if (tid == 0) {
            double total = 0.0;
            for (int w = 0; w < K::WARPS; ++w) total += dred[w];
            double* slot = T.partials + (size_t)it * C + c;
            *slot = P.accumulate ? *slot + total : total;
        }
        __syncthreads();
    }
    if constexpr (epry || gd_pupil) {
        for (int e = tid; e < R * N; e += K::THREADS) {
            const int l = e / N, j = e % N;
            const int i = C == 1 ? l : c * R + l;
            __stcg(T.pupil + i * N + j, pslab[e]);
        }
    }
    if (P.momentum && c == 0 && tid == 0) *T.counter = counter;
    if (use_tma && s_tma_failed) {
        // A stencil load that timed out may still land: let it, before exit.
        const unsigned long long t0 = global_ns();
        while (global_ns() - t0 < 1000000ull) {
        }
    }
    if (!spectral && T.object_err) {
        // Compensated accumulation: the carried error goes back into the
        // object at the end of the launch (every frame's P8 is done), so
        // whatever reads the state next sees O - E; the error restarts at zero.
        cluster_barrier<K>();
        const long long total = (long long)M * ostride / 2;
        const long long per = (total + C - 1) / C;
        const long long begin = c * per;
        const long long end = begin + per < total ? begin + per : total;
        float4* O4 = reinterpret_cast<float4*>(T.object);
        float4* E4 = reinterpret_cast<float4*>(T.object_err);
        for (long long e = begin + tid; e < end; e += K::THREADS) {
            const float4 err = __ldcg(E4 + e);
            float4 o = __ldcg(O4 + e);
            o.x -= err.x;
            o.y -= err.y;
            o.z -= err.z;
            o.w -= err.w;
            __stcg(O4 + e, o);
            __stcg(E4 + e, make_float4(0.f, 0.f, 0.f, 0.f));
        }
    }
    // Peers must not exit, nor take their next tile, while their shared
    // memory may still be addressed.
    cluster_barrier<K>();
    if (tma_capable && tid == 0) mbar_inval(&s_tma_bar);  // initialised again by the next tile
}

// Persistent frame engine: the launch has G clusters (G <= the tile count,
// chosen per tile size); cluster k reconstructs tiles k, k + G, k + 2G, ...
// of the launch, each as engine_tile.
template <int N_, int ALG, int LOSS>
__global__ void __launch_bounds__(Cfg<N_>::THREADS, Cfg<N_>::MIN_BLOCKS) engine_kernel(const EngineParams P) {
    const int clusters = (int)(gridDim.x / Cfg<N_>::C);
    for (int tile = (int)(blockIdx.x / Cfg<N_>::C); tile < P.tile_count; tile += clusters)
        engine_tile<N_, ALG, LOSS>(P, tile);
}

// Forward model (simulate): cluster f computes frame f's intensity.
template <int N_>
__global__ void __launch_bounds__(Cfg<N_>::THREADS) forward_kernel(const ForwardParams P) {
    using K = Cfg<N_>;
    constexpr int N = K::N, R = K::R, C = K::C, NA = K::NA, NB = K::NB;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    float2* field = reinterpret_cast<float2*>(smem_raw);
    float2* fld = field + K::RS;
    float2* osm = field + K::FIELD;
    float2* pslab = osm + K::STAGE;
    float2* tw = pslab + K::PSLAB;
    const int tid = threadIdx.x;
    const int f = blockIdx.x / C;
    const int c = C == 1 ? 0 : (int)(blockIdx.x % C);
    const int i_lo = C == 1 ? 0 : c * R;
    const long long ostride = P.M + (P.M & 1);
    for (int k = tid; k < 256; k += K::THREADS) tw[k] = c_tw256[k];
    load_pupil_slab<K>(pslab, P.pupil, c);
    const FrameParam fp = P.params[f];
    stage_object<K>(osm, P.object, P.M, ostride, fp, i_lo, 0, N - 1);
    __syncthreads();
    float a = 0.f, b = 0.f;
    rows_inverse<K, false>(fld, osm + (fp.lower_col & 1), tw, pslab, fp, c, i_lo, 0, N - 1, a, b);
    cluster_barrier<K>();
    if constexpr (C > 1) {
        columns_cross_inverse<K>(fld, tw, c, 0, N - 1);
        cluster_barrier<K>();
    }
    float* out = P.out + (size_t)f * N * N;
    const float* bg = P.background ? P.background + (size_t)f * P.background_stride : nullptr;
    {
        const int warp = tid >> 5, lane = tid & 31;
        const int q = R == 32 ? (warp << 4) | (lane & 15) : tid, h = R == 32 ? lane >> 4 : 0;
        float2 v[16];
        if constexpr (R == 32) column_inverse_split<K>(fld, phys<K>(q), h, tw, v);
        else column_inverse_local<K>(fld, phys<K>(q), v);
        const int ka = q / NB, kb = q % NB;
        const int x = ka + NA * kb;
#pragma unroll
        for (int k = 0; k < 16; ++k) {
            const int y = c + C * (R == 32 ? h + 2 * k : k);
            const float b0 = bg ? bg[y * N + x] : 0.f;
            out[y * N + x] = fmaf(fp.gain, cnorm2(v[k]), b0);
        }
    }
    cluster_barrier<K>();
}

// Natural (y, x) -> engine layout index within one frame.
template <class K>
FPM_DEVICE int perm_index(int y, int x) {
    const int c = y % K::C, m = y / K::C;  // CTA c holds spatial rows c + C * m
    const int ka = x % K::NA, kb = x / K::NA;
    return (c * K::R + m) * K::N + K::NB * ka + kb;
}

// Natural column x of engine-layout position t within a row: positions
// NB * ka + kb hold columns ka + NA * kb.
template <class K>
FPM_DEVICE int layout_column(int t) {
    return t / K::NB + K::NA * (t % K::NB);
}

// Natural -> engine layout, one row per block (blockDim.x == N): the row is
// read and written contiguously; the column shuffle goes through shared
// memory. Row `row` of frame f is natural row y; its engine row starts at
// (c * R + m) * N with y = c + C * m.
template <class K>
FPM_DEVICE long long layout_row_base(long long f, int y) {
    return f * K::N * K::N + (long long)((y % K::C) * K::R + y / K::C) * K::N;
}

template <int N_>
__global__ void __launch_bounds__(N_) permute_f64_kernel(const double* __restrict__ src, float* __restrict__ dst,
                                                         long long frames) {
    using K = Cfg<N_>;
    __shared__ float row[N_];
    for (long long r = blockIdx.x; r < frames * K::N; r += gridDim.x) {
        const long long f = r / K::N;
        const int y = (int)(r % K::N), t = threadIdx.x;
        row[t] = (float)src[r * K::N + t];
        __syncthreads();
        dst[layout_row_base<K>(f, y) + t] = row[layout_column<K>(t)];
        __syncthreads();
    }
}

// Engine layout -> natural order, widened to FP64: the inverse of
// permute_f64_kernel (engine position t of a row holds natural column
// layout_column(t)).
template <int N_>
__global__ void __launch_bounds__(N_) unpermute_f64_kernel(const float* __restrict__ src, double* __restrict__ dst,
                                                           long long frames) {
    using K = Cfg<N_>;
    for (long long r = blockIdx.x; r < frames * K::N; r += gridDim.x) {
        const long long f = r / K::N;
        const int y = (int)(r % K::N), t = threadIdx.x;
        dst[r * K::N + layout_column<K>(t)] = (double)src[layout_row_base<K>(f, y) + t];
    }
}

template <int N_>
__global__ void __launch_bounds__(N_) permute_u8_kernel(const uint8_t* __restrict__ src, uint8_t* __restrict__ dst,
                                                        long long frames) {
    using K = Cfg<N_>;
    __shared__ uint8_t row[N_];
    for (long long r = blockIdx.x; r < frames * K::N; r += gridDim.x) {
        const long long f = r / K::N;
        const int y = (int)(r % K::N), t = threadIdx.x;
        row[t] = src[r * K::N + t];
        __syncthreads();
        dst[layout_row_base<K>(f, y) + t] = row[layout_column<K>(t)];
        __syncthreads();
    }
}

// Weighted mean amplitude per detector pixel, nearest upsample to M x M.
// Block b of a tile handles pixels [b * 256, b * 256 + 256); a second pass
// resolves the fallback for pixels without any positive-weight sample.
constexpr int kInitBlock = 256;

template <int N_>
__global__ void init_mean_kernel(const InitTile* __restrict__ tiles, double* __restrict__ avg,
                                 double* __restrict__ partial) {
    using K = Cfg<N_>;
    constexpr int N = K::N;
    const InitTile T = tiles[blockIdx.y];
    const int chunks = gridDim.x;
    // Threads walk the engine layout (coalesced reads of every frame); each
    // writes its natural pixel's mean.
    const int idx = blockIdx.x * kInitBlock + threadIdx.x;
    __shared__ double s_amp[kInitBlock / 32], s_w[kInitBlock / 32];
    double sum = 0.0, wsum = 0.0;
    if (idx < N * N) {
        const int erow = idx / N, c = erow / K::R, m = erow % K::R;
        const int p = (c + K::C * m) * N + layout_column<K>(idx % N);  // natural pixel
        for (int f = 0; f < T.frames_count; ++f) {
            const FrameParam fp = T.params[f];
            if (fp.weight == 0.0f) continue;
            const size_t off = (size_t)f * N * N + idx;
            double amp;
            if (T.amplitude) {
                if (T.meas[off] < 0.0f) continue;
                amp = (double)T.meas[off];
            } else {
                if (T.masks && T.masks[off] == 0) continue;
                const double bg = T.background ? (double)T.background[(size_t)f * T.background_stride + idx] : 0.0;
                amp = sqrt(fmax(((double)T.meas[off] - bg) / (double)fp.gain, 0.0));
            }
            sum += (double)fp.weight * amp;
            wsum += (double)fp.weight;
        }
        avg[(size_t)blockIdx.y * N * N + p] = wsum > 0.0 ? sum / wsum : -1.0;
    }
    double a = warp_sum(sum), b = warp_sum(wsum);
    if ((threadIdx.x & 31) == 0) {
        s_amp[threadIdx.x >> 5] = a;
        s_w[threadIdx.x >> 5] = b;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double ta = 0.0, tb = 0.0;
        for (int w = 0; w < kInitBlock / 32; ++w) {
            ta += s_amp[w];
            tb += s_w[w];
        }
        partial[((size_t)blockIdx.y * chunks + blockIdx.x) * 2] = ta;
        partial[((size_t)blockIdx.y * chunks + blockIdx.x) * 2 + 1] = tb;
    }
}

template <int N_>
__global__ void init_upsample_kernel(const InitTile* __restrict__ tiles, int m, const double* __restrict__ avg,
                                     const double* __restrict__ partial, int chunks) {
    constexpr int N = N_;
    const InitTile T = tiles[blockIdx.y];
    __shared__ double s_fallback;
    if (threadIdx.x == 0) {
        double ta = 0.0, tb = 0.0;
        for (int k = 0; k < chunks; ++k) {
            ta += partial[((size_t)blockIdx.y * chunks + k) * 2];
            tb += partial[((size_t)blockIdx.y * chunks + k) * 2 + 1];
        }
        s_fallback = tb > 0.0 ? ta / tb : 0.0;
        if (!(tb > 0.0) && blockIdx.x == 0) atomicOr(T.status, 4);
    }
    __syncthreads();
    const double* a = avg + (size_t)blockIdx.y * N * N;
    const long long total = (long long)m * m;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
        const int r = (int)(e / m), col = (int)(e % m);
        const int lr = (int)((long long)r * N / m), lc = (int)((long long)col * N / m);
        double v = a[lr * N + lc];
        if (v < 0.0) v = s_fallback;
        T.scratch[e] = make_double2(v, 0.0);
    }
}

// ------------------------------------------------------------- launchers

template <int N_, class Kern, class Params>
cudaError_t launch_cluster(Kern kernel, const Params& p, int clusters, cudaStream_t s) {
    using K = Cfg<N_>;
    cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, K::SMEM_BYTES);
    if (e != cudaSuccess) return e;
    if constexpr (K::C > 8) {
        // 16-CTA clusters are beyond the portable size of 8.
        e = cudaFuncSetAttribute(kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        if (e != cudaSuccess) return e;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(clusters * K::C);
    cfg.blockDim = dim3(K::THREADS);
    cfg.dynamicSmemBytes = K::SMEM_BYTES;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = K::C;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, p);
}

// Per-size entry points; each tile size is instantiated in its own
// translation unit (engine_n32.cu ... engine_n256.cu) so they build in parallel.
// One algorithm family's engine launch (amplitude-MSE specialisation, or the
// runtime-selected loss). Instantiated per tile size; the gradient-descent
// and adaptive families live in their own translation units
// (engine_n*_gd.cu) so each size builds as two parallel halves.
template <int N_, int ALG>
cudaError_t launch_engine_alg(const EngineParams& p, int tiles, cudaStream_t s) {
    if constexpr (ALG == kAlgSpectral) {
        // Spectral AP's loss is a diagnostic: one runtime-selected variant.
        return launch_cluster<N_>(engine_kernel<N_, ALG, -1>, p, tiles, s);
    } else {
        if (p.loss == 0) return launch_cluster<N_>(engine_kernel<N_, ALG, 0>, p, tiles, s);
        return launch_cluster<N_>(engine_kernel<N_, ALG, -1>, p, tiles, s);
    }
}

#define FPM_ENGINE_SECOND_HALF(N, SPEC)                                                                  \
    SPEC template cudaError_t launch_engine_alg<N, kAlgGradient>(const EngineParams&, int, cudaStream_t); \
    SPEC template cudaError_t launch_engine_alg<N, kAlgGradientTruncated>(const EngineParams&, int,      \
                                                                          cudaStream_t);               \
    SPEC template cudaError_t launch_engine_alg<N, kAlgLocalAdaptive>(const EngineParams&, int, cudaStream_t); \
    SPEC template cudaError_t launch_engine_alg<N, kAlgGradientPupil>(const EngineParams&, int, cudaStream_t); \
    SPEC template cudaError_t launch_engine_alg<N, kAlgSpectral>(const EngineParams&, int, cudaStream_t);    \
    SPEC template cudaError_t launch_engine_alg<N, kAlgGlobalCal>(const EngineParams&, int, cudaStream_t);   \
    SPEC template cudaError_t launch_engine_alg<N, kAlgEpryCal>(const EngineParams&, int, cudaStream_t);

template <int N_>
struct EngineEntry {
    template <int ALG>
    static cudaError_t engine_alg(const EngineParams& p, int tiles, cudaStream_t s) {
        return launch_engine_alg<N_, ALG>(p, tiles, s);
    }

    static cudaError_t engine(const EngineParams& p, int tiles, cudaStream_t s) {
        switch (p.alg) {
            case kAlgLocal: return engine_alg<kAlgLocal>(p, tiles, s);
            case kAlgRpie: return engine_alg<kAlgRpie>(p, tiles, s);
            case kAlgGlobal: return engine_alg<kAlgGlobal>(p, tiles, s);
            case kAlgEpry: return engine_alg<kAlgEpry>(p, tiles, s);
            case kAlgGlobalCal: return engine_alg<kAlgGlobalCal>(p, tiles, s);
            case kAlgEpryCal: return engine_alg<kAlgEpryCal>(p, tiles, s);
            case kAlgGradient: return engine_alg<kAlgGradient>(p, tiles, s);
            case kAlgGradientTruncated: return engine_alg<kAlgGradientTruncated>(p, tiles, s);
            case kAlgLocalAdaptive: return engine_alg<kAlgLocalAdaptive>(p, tiles, s);
            case kAlgGradientPupil: return engine_alg<kAlgGradientPupil>(p, tiles, s);
            case kAlgSpectral: return engine_alg<kAlgSpectral>(p, tiles, s);
            default: return cudaErrorInvalidValue;
        }
    }

    // Clusters of the frame engine that can be resident at once on the
    // current device (every family shares the shape and the register cap).
    static cudaError_t max_active_clusters(int* count) {
        using K = Cfg<N_>;
        auto kernel = engine_kernel<N_, kAlgRpie, 0>;
        cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, K::SMEM_BYTES);
        if (e != cudaSuccess) return e;
        if constexpr (K::C > 8) {
            e = cudaFuncSetAttribute(kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
            if (e != cudaSuccess) return e;
        }
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(K::C);
        cfg.blockDim = dim3(K::THREADS);
        cfg.dynamicSmemBytes = K::SMEM_BYTES;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = K::C;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        return cudaOccupancyMaxActiveClusters(count, kernel, &cfg);
    }

    static cudaError_t forward(const ForwardParams& p, cudaStream_t s) {
        return launch_cluster<N_>(forward_kernel<N_>, p, p.frame_count, s);
    }

    // One block of N threads per frame row (grid-strided over the rows).
    static int permute_blocks(long long frames) {
        const long long rows = frames * N_;
        return (int)(rows < 65536 ? rows : 65536);
    }

    static cudaError_t permute_f64(const double* src, float* dst, long long frames, cudaStream_t s) {
        if (frames <= 0) return cudaSuccess;
        permute_f64_kernel<N_><<<permute_blocks(frames), N_, 0, s>>>(src, dst, frames);
        return cudaGetLastError();
    }

    static cudaError_t unpermute_f64(const float* src, double* dst, long long frames, cudaStream_t s) {
        if (frames <= 0) return cudaSuccess;
        unpermute_f64_kernel<N_><<<permute_blocks(frames), N_, 0, s>>>(src, dst, frames);
        return cudaGetLastError();
    }

    static cudaError_t permute_u8(const uint8_t* src, uint8_t* dst, long long frames, cudaStream_t s) {
        if (frames <= 0) return cudaSuccess;
        permute_u8_kernel<N_><<<permute_blocks(frames), N_, 0, s>>>(src, dst, frames);
        return cudaGetLastError();
    }

    static cudaError_t init(int m, const InitTile* tiles, int count, double* avg, double* partial, cudaStream_t s) {
        const int chunks = (N_ * N_ + kInitBlock - 1) / kInitBlock;
        init_mean_kernel<N_><<<dim3(chunks, count), kInitBlock, 0, s>>>(tiles, avg, partial);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        const long long total = (long long)m * m;
        const int blocks = (int)((total + 255) / 256 < 1024 ? (total + 255) / 256 : 1024);
        init_upsample_kernel<N_><<<dim3(blocks, count), 256, 0, s>>>(tiles, m, avg, partial, chunks);
        return cudaGetLastError();
    }
};

}  // namespace fpm
