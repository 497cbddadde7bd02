// Single-CTA frame engine for 256 x 256 tiles of the fixed-pupil projection
// families (AP, FPIE/mPIE, EPRY without pupil recovery): the per-frame update
// of src/algorithms/common.rs:57-306 for many independent tiles.
//
// One CTA of 512 threads owns a tile and walks its frames in the reference's
// sequential order. The 2-D transforms pass through a per-CTA field scratch
// in global memory (256 x 256 complex64, rows indexed by centred patch row;
// only the pupil's rows are ever touched, so it stays in L2), and every phase
// boundary is a block barrier: no cluster barriers or distributed shared
// memory exchanges. Per frame:
//
//   A  support rows: bilinear patch * pupil (ifftshifted), row inverse
//      transform 16 x 16 (registers, a half-warp transpose in shared memory)
//      -> scratch rows, positions t = 16 ka + kb holding column ka + 16 kb
//   B  32 positions at a time: column inverse 16 x 16 (the block transposes
//      through shared memory), amplitude projection against the measurement
//      (the engine layout, so reads are contiguous), column forward 16 x 16
//      -> scratch, support rows only
//   C  row forward transform, fftshift, the correction U (local / rPIE /
//      global denominator) into a per-warp ring of U rows in shared memory,
//      and the exact bilinear adjoint of U added into the object
//      (src/model/crop.rs:188-255); each warp owns a band of object rows
//
// The transforms, twiddles and per-pixel arithmetic are the cluster engine's
// (engine_impl.cuh), term by term and in the same order; only the place a
// value waits between two steps differs. The measurement layout is the
// cluster engine's for 256-point tiles, so problems upload once for both.
#include "engine_impl.cuh"

namespace fpm {
namespace {

constexpr int kL2N = 256;
// 512 threads per CTA, one CTA per SM (128 registers per thread). Two
// 256-thread CTAs per SM (kL2Threads = 256, 16-position blocks in phase B)
// measured the same SM time per tile and a slower tile mix on GB300.
constexpr int kL2Threads = 512;
constexpr int kL2PerSm = 512 / kL2Threads;     // resident CTAs per SM (registers: 128 per thread)
constexpr int kL2Warps = kL2Threads / 32;
constexpr int kL2Pos = kL2Threads / 16;        // phase B: positions per block (one thread per digit and position)
constexpr int kL2Stage = 16 * 16 * kL2Pos;     // one column-stage buffer: [16][16][positions]
constexpr int kL2Tp = 17;                      // transpose row stride (float2): conflict-free rows and columns
constexpr int kL2HalfBuf = 16 * kL2Tp;         // one half-warp's 16 x 16 transpose buffer
constexpr int kL2Slot = 16 * kL2Tp;            // one ring row: N = 256 values of U, or a transpose
constexpr int kL2CtaOfN = Cfg<kL2N>::C;        // objective partial slots per iteration for this size
// Work region: the two column stages of phase B; the 32 half-warp
// transposes of phase A; each warp's ring of three U rows in phase C (whose
// transposes use the ring row being replaced).
constexpr int kL2Rings = kL2Warps * 3 * kL2Slot;
static_assert(kL2Slot >= kL2N, "a ring row holds a row of U");
constexpr int kL2Region = 2 * kL2Stage > kL2Rings ? 2 * kL2Stage : kL2Rings;
static_assert(2 * kL2Warps * kL2HalfBuf <= kL2Region, "phase A transposes fit the work region");
// tw[256] + work region + pupil spans [N] + per-warp FP64 partials.
constexpr int kL2SmemBytes = (256 + kL2Region) * 8 + kL2N * 8 + kL2Warps * 8;

// Preferred shared-memory carveout (percent of the 228 KB maximum): the
// resident CTAs' dynamic and static shared memory plus the 1 KB reserved per CTA.
constexpr int kL2Carveout = (kL2PerSm * (kL2SmemBytes + 1024 + 1024) * 100 + 228 * 1024 - 1) / (228 * 1024);

// Element (r, c) of a 16 x 16 transpose buffer.
FPM_DEVICE constexpr int tpos(int r, int c) { return r * kL2Tp + c; }

// Patch * pupil at the 16 ifftshifted columns j = (16 na + hl + N/2) mod N
// of centred row i, the bilinear stencil read from the object (o0: row
// lower_row + i from column lower_col). UNIT: the pupil is 1 on [sp.x, sp.y]
// and 0 elsewhere, so the product is the patch or zero (the values a general
// pupil's complex product gives). GUARD: cells past the grid read as zero
// (the frame's stencil crosses the grid edge).
template <bool UNIT, bool GUARD>
FPM_DEVICE void gather_row(float2 (&v)[16], const float2* __restrict__ o0, long long ostride, int hl, int col_room,
                           bool row0, bool row1, int2 sp, const float2* __restrict__ prow, float w00, float w01,
                           float w10, float w11) {
    constexpr int N = kL2N;
#pragma unroll
    for (int na = 0; na < 16; ++na) {
        const int j = (16 * na + hl + N / 2) & (N - 1);
        const float2 z = make_float2(0.f, 0.f);
        float2 a00, a01, a10, a11;
        if constexpr (GUARD) {
            const bool col0 = j < col_room, col1 = j + 1 < col_room;
            a00 = row0 && col0 ? o0[j] : z;
            a01 = row0 && col1 ? o0[j + 1] : z;
            a10 = row1 && col0 ? o0[j + ostride] : z;
            a11 = row1 && col1 ? o0[j + ostride + 1] : z;
        } else {
            a00 = o0[j];
            a01 = o0[j + 1];
            a10 = o0[j + ostride];
            a11 = o0[j + ostride + 1];
        }
        float2 pt = cscale(a00, w00);
        pt = cfma(w01, a01, pt);
        pt = cfma(w10, a10, pt);
        pt = cfma(w11, a11, pt);
        if constexpr (UNIT) {
            v[na] = (unsigned)(j - sp.x) <= (unsigned)(sp.y - sp.x) ? pt : z;
        } else {
            v[na] = cmul(pt, __ldg(prow + j));
        }
    }
}

// One mPIE momentum event over the whole object (src/algorithms/common.rs:
// 308-387): velocity = friction * velocity + object - anchor, object +=
// feedback * velocity, anchor = object. Out of line, so that its registers
// do not add to the frame loop's. True when a value became non-finite.
__device__ __noinline__ bool momentum_event(float4* __restrict__ O4, float4* __restrict__ V4, float4* __restrict__ A4,
                                            float friction, float feedback, long long total, int tid) {
    bool bad = false;
    constexpr int U = 4;
    for (long long e0 = tid; e0 < total; e0 += (long long)kL2Threads * U) {
        float4 o[U], v[U], a[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const long long e = e0 + (long long)u * kL2Threads;
            if (e < total) {
                o[u] = O4[e];
                v[u] = V4[e];
                a[u] = A4[e];
            }
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const long long e = e0 + (long long)u * kL2Threads;
            if (e < total) {
                float4 nv, no;
                nv.x = fmaf(friction, v[u].x, o[u].x - a[u].x);
                nv.y = fmaf(friction, v[u].y, o[u].y - a[u].y);
                nv.z = fmaf(friction, v[u].z, o[u].z - a[u].z);
                nv.w = fmaf(friction, v[u].w, o[u].w - a[u].w);
                if (feedback == 0.f) {
                    no = o[u];
                } else {
                    no.x = fmaf(feedback, nv.x, o[u].x);
                    no.y = fmaf(feedback, nv.y, o[u].y);
                    no.z = fmaf(feedback, nv.z, o[u].z);
                    no.w = fmaf(feedback, nv.w, o[u].w);
                }
                bad |= !isfinite(nv.x) || !isfinite(nv.y) || !isfinite(nv.z) || !isfinite(nv.w) ||
                       !isfinite(no.x) || !isfinite(no.y) || !isfinite(no.z) || !isfinite(no.w);
                V4[e] = nv;
                O4[e] = no;
                A4[e] = no;
            }
        }
    }
    return bad;
}

template <int ALG, int LOSS, bool UNIT>
FPM_DEVICE void engine_l2_tile(const EngineParams& P, const int tile) {
    constexpr int N = kL2N;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    float2* const tw = reinterpret_cast<float2*>(smem_raw);
    float2* const S = tw + 256;
    float2* const S2 = S + kL2Stage;
    float2* const U = S;
    int2* const spans = reinterpret_cast<int2*>(S + kL2Region);
    double* const dred = reinterpret_cast<double*>(spans + N);
    __shared__ TileDesc s_tile;
    __shared__ FrameParam s_frame;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int half = lane >> 4, hl = lane & 15;
    float2* const tb = S + (warp * 2 + half) * kL2HalfBuf;  // phase A
    float2* const G = P.field_scratch + (size_t)blockIdx.x * N * N;

    if (tid == 0) s_tile = P.tiles[tile];
    for (int k = tid; k < 256; k += kL2Threads) tw[k] = c_tw256[k];
    __syncthreads();
    const TileDesc& T = s_tile;
    // A unit pupil (exactly 1 on one column interval per row, 0 elsewhere)
    // is read from its row spans (UNIT launches: every tile has one).
    for (int k = tid; k < N; k += kL2Threads) spans[k] = UNIT ? T.pupil_span[k] : make_int2(0, -1);
    const int M = T.M;
    const long long ostride = M + (M & 1);
    const int row_lo = T.row_lo, row_hi = T.row_hi;
    const int n_rows = row_hi - row_lo + 1;  // empty support: n_rows <= 0
    const float eps = opaque((float)P.eps);
    const float inv_n2 = 1.0f / (float)(N * N);
    const double max_p2 = T.max_pupil_power;
    const float inv_global = opaque((float)(1.0 / (max_p2 + P.eps)));
    const float rpie_a = opaque((float)(1.0 - P.alpha)), rpie_b = opaque((float)(P.alpha * max_p2 + P.eps));
    // The correction's denominator where a unit pupil is 1 (|P|^2 = 1).
    const float inv_one = opaque(ALG == kAlgLocal ? 1.0f / (1.0f + eps)
                                 : ALG == kAlgRpie ? 1.0f / fmaf(rpie_a, 1.0f, rpie_b)
                                                   : inv_global);
    int counter = P.momentum ? *T.counter : 0;
    double loss_acc = 0.0;
    __syncthreads();

    for (int it = P.it_begin; it < P.it_end; ++it) {
        const int steps = T.frame_count;
        const int step_begin = P.frame_end > 0 ? P.frame_begin : 0;
        const int step_end = P.frame_end > 0 ? min(P.frame_end, steps) : steps;
        for (int idx = step_begin; idx < step_end; ++idx) {
            const int f = T.order ? __ldg(T.order + idx) : idx;
            if (tid == 0) s_frame = T.params[f];
            if (tid < 16 && idx + 1 < step_end) {
                // The next frame's measurement goes to L2 behind this frame.
                const int f1 = T.order ? __ldg(T.order + idx + 1) : idx + 1;
                prefetch_l2(T.meas + (size_t)f1 * N * N + (size_t)tid * (N * N / 16), N * N / 16 * sizeof(float));
            }
            __syncthreads();
            const FrameParam& fp = s_frame;
            if (fp.weight == 0.0f) {
                __syncthreads();
                continue;
            }

            // A: row inverse transforms of the support rows into the scratch.
            // Frames whose stencil lies inside the grid skip the edge checks.
            const bool in_grid = fp.lower_row + row_hi + 1 < M && fp.lower_col + N < M;
            for (int p = warp; 2 * p < n_rows; p += kL2Warps) {
                const int i = row_lo + 2 * p + half;
                const bool live = i <= row_hi;
                float2 v[16];
                if (live) {
                    const int gr = fp.lower_row + i;
                    const float2* o0 = T.object + (long long)gr * ostride + fp.lower_col;
                    const float2* prow = UNIT ? nullptr : T.pupil + i * N;
                    const float w00 = fp.w00, w01 = fp.w01, w10 = fp.w10, w11 = fp.w11;
                    if (in_grid)
                        gather_row<UNIT, false>(v, o0, ostride, hl, 0, true, true, spans[i], prow, w00, w01, w10, w11);
                    else
                        gather_row<UNIT, true>(v, o0, ostride, hl, M - fp.lower_col, gr < M, gr + 1 < M, spans[i],
                                               prow, w00, w01, w10, w11);
                    dft_reg<16, true>(v);
#pragma unroll
                    for (int ka = 0; ka < 16; ++ka) tb[tpos(ka, hl)] = twiddle_smem<true>(v[ka], tw, hl * ka);
                }
                __syncwarp();
                if (live) {
#pragma unroll
                    for (int nb = 0; nb < 16; ++nb) v[nb] = tb[tpos(hl, nb)];
                    dft_reg<16, true>(v);  // v[kb]: column hl + 16 kb, position 16 hl + kb
                }
                __syncwarp();
                if (live) {
#pragma unroll
                    for (int kb = 0; kb < 16; ++kb) tb[tpos(hl, kb)] = v[kb];
                }
                __syncwarp();
                if (live) {
                    float2* g = G + (size_t)i * N;
#pragma unroll
                    for (int k = 0; k < 16; ++k) g[16 * k + hl] = tb[tpos(k, hl)];
                }
                __syncwarp();
            }
            __syncthreads();

            // B: columns, kL2Pos positions t at a time; thread (d, pos) with
            // d = tid / kL2Pos. Stage 1: d = natural row low digit l,
            // register = high digit; stage 2: d = k1, register m = spatial
            // row k1 + 16 m (the engine layout's row 16 k1 + m); the forward
            // transform mirrors it.
            {
                const float gain = fp.gain;
                float frame_loss = 0.f;
                const int d = tid / kL2Pos, pos = tid % kL2Pos;
#pragma unroll 1
                for (int blk = 0; blk < N / kL2Pos; ++blk) {
                    const int t = kL2Pos * blk + pos;
                    float mreg[16];
                    {
                        const float* mrow = T.meas + (size_t)f * N * N + (size_t)(16 * d) * N + t;
#pragma unroll
                        for (int m = 0; m < 16; ++m) mreg[m] = __ldcs(mrow + (size_t)m * N);
                    }
                    float2 v[16];
#pragma unroll
                    for (int nc = 0; nc < 16; ++nc) {
                        const int i = (16 * nc + d + N / 2) & (N - 1);
                        v[nc] = i >= row_lo && i <= row_hi ? G[(size_t)i * N + t] : make_float2(0.f, 0.f);
                    }
                    dft_reg<16, true>(v);
#pragma unroll
                    for (int k1 = 0; k1 < 16; ++k1)
                        S[(k1 * 16 + d) * kL2Pos + pos] = twiddle_smem<true>(v[k1], tw, d * k1);
                    __syncthreads();
#pragma unroll
                    for (int l = 0; l < 16; ++l) v[l] = S[(d * 16 + l) * kL2Pos + pos];
                    dft_reg<16, true>(v);
                    // Amplitude projection: the forward transform takes psi' - psi
                    // (masked pixels contribute zero).
#pragma unroll
                    for (int m = 0; m < 16; ++m) {
                        const float a = mreg[m];
                        const float intrinsic = cnorm2(v[m]);
                        const float r = rsqrtf(fmaxf(intrinsic, 1.17549435e-38f));
                        const float s_amp = intrinsic * r;
                        if (a >= 0.f) {
                            if constexpr (LOSS == 0) {
                                const float dd = s_amp - a;
                                frame_loss = fmaf(dd, dd, frame_loss);
                            } else {
                                frame_loss += point_loss<LOSS>(gain * intrinsic, gain * a * a, P.loss);
                            }
                            v[m] = intrinsic > eps ? cscale(v[m], fmaf(a, r, -1.f)) : make_float2(a - v[m].x, -v[m].y);
                        } else {
                            v[m] = make_float2(0.f, 0.f);
                        }
                    }
                    dft_reg<16, false>(v);
#pragma unroll
                    for (int b = 0; b < 16; ++b)
                        S2[(b * 16 + d) * kL2Pos + pos] = twiddle_smem<false>(v[b], tw, d * b);
                    __syncthreads();
#pragma unroll
                    for (int k1 = 0; k1 < 16; ++k1) v[k1] = S2[(d * 16 + k1) * kL2Pos + pos];
                    dft_reg<16, false>(v);
#pragma unroll
                    for (int j1 = 0; j1 < 16; ++j1) {
                        const int i = (16 * j1 + d + N / 2) & (N - 1);
                        if (i >= row_lo && i <= row_hi) G[(size_t)i * N + t] = v[j1];
                    }
                }
                if (LOSS == 0) frame_loss *= gain;
                loss_acc += (double)frame_loss * fp.loss_scale;
            }
            __syncthreads();

            // C: row forward transforms, fftshift, the correction U and its
            // bilinear adjoint into the object. The object rows the frame
            // changes are split into one contiguous band per warp; a warp
            // walks U rows a - 1 .. b - 1 of its band [a, b) in pairs (one
            // row per half-warp) through a ring of three U rows in shared
            // memory, so object row r finds U rows r and r - 1 there (rows
            // outside the support are zero).
            {
                const float scale = opaque((float)((double)fp.weight * P.object_step));
                const int rows8 = N + fp.has_upper_row;
                const int cols8 = N + fp.has_upper_col;
                const int r_first = max(row_lo, 0), r_last = min(row_hi + 1, rows8 - 1);
                const int per = (r_last - r_first + kL2Warps) / kL2Warps;  // ceil(count / warps); count may be <= 0
                const int a = r_first + warp * per, b = min(a + per, r_last + 1);
                float2* const ring = U + warp * 3 * kL2Slot;
                for (int k = a - 1; k < b; k += 2) {
                    const int i = k + half;  // the U row of this half-warp (>= -1)
                    float2* const slot = ring + ((i + 3) % 3) * kL2Slot;
                    const bool need = i < b;
                    const bool live = need && i >= row_lo && i <= row_hi;
                    float2 v[16];
                    if (live) {
                        const float4* g4 = reinterpret_cast<const float4*>(G + (size_t)i * N + 16 * hl);
#pragma unroll
                        for (int q = 0; q < 8; ++q) {
                            const float4 w = g4[q];
                            v[2 * q] = make_float2(w.x, w.y);
                            v[2 * q + 1] = make_float2(w.z, w.w);
                        }
                        dft_reg<16, false>(v);
#pragma unroll
                        for (int jb = 0; jb < 16; ++jb) slot[tpos(jb, hl)] = twiddle_smem<false>(v[jb], tw, hl * jb);
                    }
                    __syncwarp();
                    if (live) {
#pragma unroll
                        for (int ka = 0; ka < 16; ++ka) v[ka] = slot[tpos(hl, ka)];
                    }
                    __syncwarp();  // the slot's transpose is read before U replaces it
                    if (live) {
                        dft_reg<16, false>(v);
                        const int2 sp = spans[i];
#pragma unroll
                        for (int ja = 0; ja < 16; ++ja) {
                            const int j = (16 * ja + hl + N / 2) & (N - 1);
                            const float2 psi = cscale(v[ja], inv_n2);
                            float2 u;
                            if constexpr (UNIT) {
                                // conj(P) * psi / den with P = 1 inside the span, 0 outside.
                                u = (unsigned)(j - sp.x) <= (unsigned)(sp.y - sp.x) ? cscale(psi, inv_one)
                                                                                    : make_float2(0.f, 0.f);
                            } else {
                                const float2 pv = __ldg(T.pupil + i * N + j);
                                const float pw = cnorm2(pv);
                                float inv_den;
                                if constexpr (ALG == kAlgLocal)
                                    inv_den = 1.0f / (pw + eps);
                                else if constexpr (ALG == kAlgRpie)
                                    inv_den = 1.0f / fmaf(rpie_a, pw, rpie_b);
                                else
                                    inv_den = inv_global;
                                u = cscale(cmulc(psi, pv), inv_den);
                            }
                            slot[j] = u;
                        }
                    } else if (need) {
#pragma unroll
                        for (int m = 0; m < 16; ++m) slot[16 * m + hl] = make_float2(0.f, 0.f);
                    }
                    __syncwarp();
                    // Object row i from U rows i (this slot) and i - 1.
                    if (i >= a && i < b) {
                        const float2* u0 = slot;
                        const float2* u1 = ring + ((i + 2) % 3) * kL2Slot;
                        float2* grow = T.object + (long long)(fp.lower_row + i) * ostride + fp.lower_col;
                        const float w00 = fp.w00, w01 = fp.w01, w10 = fp.w10, w11 = fp.w11;
#pragma unroll
                        for (int h = 0; h < 2; ++h) {
                            // Columns 16 m + hl for m in [9h, 9h + 9) (m <= 16).
                            float2 base[9];
#pragma unroll
                            for (int q = 0; q < 9; ++q) {
                                const int j = 16 * (9 * h + q) + hl;
                                base[q] = 9 * h + q < 17 && j < cols8 ? grow[j] : make_float2(0.f, 0.f);
                            }
#pragma unroll
                            for (int q = 0; q < 9; ++q) {
                                const int j = 16 * (9 * h + q) + hl;
                                if (9 * h + q < 17 && j < cols8) {
                                    const float2 z = make_float2(0.f, 0.f);
                                    const float2 a0 = j < N ? u0[j] : z;
                                    const float2 b0 = j >= 1 ? u0[j - 1] : z;
                                    const float2 d0 = j < N ? u1[j] : z;
                                    const float2 d1 = j >= 1 ? u1[j - 1] : z;
                                    float2 acc = cscale(a0, w00);
                                    acc = cfma(w01, b0, acc);
                                    acc = cfma(w10, d0, acc);
                                    acc = cfma(w11, d1, acc);
                                    grow[j] = cfma(scale, acc, base[q]);
                                }
                            }
                        }
                    }
                    __syncwarp();  // the ring rows are read before the next pair overwrites two of them
                }
            }
            __syncthreads();

            // mPIE momentum event (src/algorithms/common.rs:308-387).
            if (P.momentum) {
                counter += 1;
                if (counter >= P.interval) {
                    counter = 0;
                    // float4 = two complex values
                    const bool bad = momentum_event(reinterpret_cast<float4*>(T.object), reinterpret_cast<float4*>(T.velocity),
                                                    reinterpret_cast<float4*>(T.anchor), P.friction, P.feedback,
                                                    (long long)M * ostride / 2, tid);
                    if (bad) atomicOr(T.status, 1);
                    __syncthreads();
                }
            }
        }
        // Objective partial of this iteration: the whole tile in slot 0 of
        // the size's per-CTA slots (the host sums the slots).
        const double s = warp_sum(loss_acc);
        loss_acc = 0.0;
        if (lane == 0) dred[warp] = s;
        __syncthreads();
        if (tid == 0) {
            double total = 0.0;
            for (int w = 0; w < kL2Warps; ++w) total += dred[w];
            double* slot = T.partials + (size_t)it * kL2CtaOfN;
            slot[0] = P.accumulate ? slot[0] + total : total;
            if (!P.accumulate)
                for (int r = 1; r < kL2CtaOfN; ++r) slot[r] = 0.0;
        }
        __syncthreads();
    }
    if (P.momentum && tid == 0) *T.counter = counter;
    __syncthreads();  // the descriptors in shared memory are rewritten by the next tile
}

template <int ALG, int LOSS, bool UNIT>
__global__ void __launch_bounds__(kL2Threads, kL2PerSm) engine_l2_kernel(const EngineParams P) {
    for (int tile = blockIdx.x; tile < P.tile_count; tile += gridDim.x) engine_l2_tile<ALG, LOSS, UNIT>(P, tile);
}

template <int ALG, int LOSS, bool UNIT>
cudaError_t launch_l2(const EngineParams& p, int ctas, cudaStream_t s) {
    auto kernel = engine_l2_kernel<ALG, LOSS, UNIT>;
    cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kL2SmemBytes);
    if (e != cudaSuccess) return e;
    // The smallest shared-memory carveout that holds the CTA, so the rest of
    // the SM's 256 KB stays L1 for the stencil reads and register spills.
    e = cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout, kL2Carveout);
    if (e != cudaSuccess) return e;
    kernel<<<ctas, kL2Threads, kL2SmemBytes, s>>>(p);
    return cudaGetLastError();
}

template <int ALG>
cudaError_t launch_l2_alg(const EngineParams& p, int ctas, cudaStream_t s) {
    if (p.unit_pupils) return p.loss == 0 ? launch_l2<ALG, 0, true>(p, ctas, s) : launch_l2<ALG, -1, true>(p, ctas, s);
    return p.loss == 0 ? launch_l2<ALG, 0, false>(p, ctas, s) : launch_l2<ALG, -1, false>(p, ctas, s);
}

}  // namespace

bool engine_l2_supported(int n, int alg) {
    return n == kL2N && (alg == kAlgLocal || alg == kAlgRpie || alg == kAlgGlobal);
}

size_t engine_l2_scratch_bytes(int n) { return (size_t)n * n * sizeof(float2); }

cudaError_t launch_engine_l2(int n, const EngineParams& p, int ctas, cudaStream_t s) {
    if (n != kL2N || ctas <= 0 || p.field_scratch == nullptr) return cudaErrorInvalidValue;
    switch (p.alg) {
        case kAlgLocal: return launch_l2_alg<kAlgLocal>(p, ctas, s);
        case kAlgRpie: return launch_l2_alg<kAlgRpie>(p, ctas, s);
        case kAlgGlobal: return launch_l2_alg<kAlgGlobal>(p, ctas, s);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t engine_l2_max_active_ctas(int n, int* count) {
    if (n != kL2N) return cudaErrorInvalidValue;
    auto kernel = engine_l2_kernel<kAlgRpie, 0, true>;
    cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kL2SmemBytes);
    if (e != cudaSuccess) return e;
    int per_sm = 0, device = 0, sms = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kL2Threads, kL2SmemBytes);
    if (e != cudaSuccess) return e;
    e = cudaGetDevice(&device);
    if (e != cudaSuccess) return e;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    if (e != cudaSuccess) return e;
    *count = per_sm * sms;
    return cudaSuccess;
}

}  // namespace fpm
