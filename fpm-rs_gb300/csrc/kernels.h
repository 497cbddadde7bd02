// Internal interface between the host runtime (runtime.cpp) and the device
// kernels (engine.cu, grid.cu). Not part of the public C ABI.
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <mutex>

struct fpm_context;

namespace fpm {

// Per-frame constants, computed once per problem on the host in FP64 and
// rounded to float. The bilinear stencil follows interpolation_axis
// (src/model/crop.rs:266-313): rows lower_row .. lower_row + N (the last one
// only when the row fraction is non-zero), likewise for columns.
struct FrameParam {
    int lower_row, lower_col;
    int has_upper_row, has_upper_col;
    float w00, w01, w10, w11;  // (lower,lower) (lower,upper) (upper,lower) (upper,upper)
    float weight;              // measurement frame weight; 0 skips the frame
    float gain;                // frame gain, > 0
    float valid_scale;         // N*N / unmasked pixel count
    float pad;
    double loss_scale;         // weight / unmasked pixel count
};

// One virtual step of narrowband spectral AP (src/algorithms/spectral.rs:
// 182-271). An exposure with K coherent modes takes K evaluation steps (the
// detector field of mode k from the pre-exposure objects into scratch slot k,
// its weighted intensity into the prediction) and then the K updates (the
// shared amplitude ratio, forward transform and local-denominator correction
// into the mode's stored object), last mode first: the last evaluation step
// also updates its own mode, so an exposure takes 2K - 1 steps. The update
// order changes only the summation order into a shared object.
struct SpectralStep {
    FrameParam frame;     // the mode's crop and bilinear weights
    int exposure;         // measurement frame
    int object, channel;  // stored object and channel pupil
    int update;           // 0: evaluate, 1: update, 2: evaluate and update (the exposure's last mode)
    int slot;             // mode position within the exposure
    int first_update;     // 1 on the exposure's first update step, which adds its loss
    float mode_weight;    // effective intensity weight of the mode
    float update_scale;   // frame weight * mode weight / exposure weight sum
    float gain;           // effective detector gain of the exposure, > 0
    float background;     // scalar exposure background
    float inv_weight_sum; // 1 / exposure weight sum (fill of dark pixels)
    float pad;
    double loss_scale;    // frame weight / unmasked pixels
};
// Steps are copied to shared memory in 16-byte pieces.
static_assert(sizeof(SpectralStep) % 16 == 0, "SpectralStep must be a whole number of 16-byte chunks");

// One reconstruction tile: device pointers into its resident buffers.
struct TileDesc {
    float2* object;            // M*M centred spectrum (state)
    float2* pupil;             // N*N state pupil
    const uint8_t* support;    // N*N
    const float* meas;         // frames * N*N, engine-permuted layout
    const uint8_t* masks;      // same layout, or null
    const float* background;   // engine-permuted, or null
    long long background_stride;  // floats between frames (0: one shared image)
    const FrameParam* params;  // [frame_count]
    // Tensor map of `object` for TMA staging of the stencil (256-point tiles;
    // viewed as [M rows][MS / 2 column pairs][4 floats]), or null.
    const void* omap;
    const int* order;          // [frame_count] schedule, or null for sequential
    float2* velocity;          // mPIE, M*M
    float2* anchor;            // mPIE, M*M
    float2* gradient;          // mini-batch gradient descent: M*M accumulator, zero between batches
    // Compensated accumulation (null when off): the running rounding error of
    // the object (or, with mini-batches, of the gradient accumulator) under
    // Kahan summation of the frame updates, M*M complex64, zero at the start.
    float2* object_err;
    float2* gradient_err;
    float2* pupil_gradient;    // gradient descent with pupil recovery: N*N accumulator, zero between batches
    double* partials;          // [iterations * cluster] objective partial sums
    int* counter;              // mPIE effective frames since the last event
    int* status;               // bits: 1 non-finite momentum, 4 no valid data, 8 gauge, 16 truncation statistic,
                               // 32 adaptive pass objective, 64 non-finite recovered pupil, 128 non-finite
                               // regulariser step
    int M, frame_count;
    double max_pupil_power;    // max(max |P|^2, eps) for fixed-pupil algorithms, FP64
    int amplitude;             // 1: meas holds sqrt(max(I / gain, 0)), -1 where masked; no masks or background
    double weight_sum;         // sum of frame weights: the objective's denominator
    // Centred pupil rows [row_lo, row_hi] that hold a non-zero pupil value.
    // With a fixed pupil every other row of psi = P * patch is zero and the
    // correction U there is zero, so the engine skips those rows (EPRY,
    // whose pupil evolves, uses the full range).
    int row_lo, row_hi;
    // Unit pupil: per centred row the column interval [x, y] where the pupil
    // is exactly 1 (0 elsewhere; empty rows hold x > y), or null when the
    // pupil has any other value. Read by the single-CTA engine.
    const int2* pupil_span;
    // Spectral AP: objects are consecutive M x (M + M % 2) grids from
    // `object`, channel pupils consecutive N x N grids from `pupil`.
    const SpectralStep* steps;  // [step_count] per pass
    int step_count;
    float2* mode_fields;        // [modes per exposure][N*N] fields, engine layout
    float* prediction;          // N*N weighted intensity sum, engine layout
};

// EPRY frame-gain and background recovery state of one tile: gains
// [frames] and backgrounds [frames][N * N] (engine layout). Kept apart from
// TileDesc, which every CTA holds in shared memory.
struct TileRecovery {
    double* gain_state;
    float* bg_state;
};

// Frame-engine kernel families, fixed at compile time so each instantiation
// carries only its own update code: AP (local |P|^2 denominator), FPIE/mPIE
// (rPIE blend), EPRY without and with pupil recovery (global max |P|^2), and
// the Wirtinger gradient.
enum EngineAlg {
    kAlgLocal = 0,
    kAlgRpie = 1,
    kAlgGlobal = 2,
    kAlgEpry = 3,
    kAlgGradient = 4,
    kAlgGradientTruncated = 5,  // gradient descent with the Poisson truncation gate
    kAlgLocalAdaptive = 6,      // AP with the adaptive step controller
    kAlgGradientPupil = 7,      // gradient descent with pupil recovery
    kAlgSpectral = 8,           // narrowband spectral AP over multi-mode exposures
    kAlgGlobalCal = 9,          // EPRY (fixed pupil) with frame-gain / background recovery
    kAlgEpryCal = 10,           // EPRY with pupil and frame-gain / background recovery
};

struct EngineParams {
    const TileDesc* tiles;
    int tile_count;            // tiles of the launch (its clusters walk them, see engine_kernel)
    int alg;
    // Step sizes, the rPIE blend and epsilon in FP64: per-frame scales and
    // denominator constants are formed in FP64 and rounded once to float.
    double alpha, eps, object_step, pupil_step;
    int constrain_pupil;
    int momentum, interval;
    float friction, feedback;
    int loss;
    int it_begin, it_end;
    int gd_batch;              // gradient descent frames per mini-batch (1: update after every frame)
    float trunc_threshold;     // gradient descent Poisson truncation threshold (0: off)
    double progress_threshold, reduction_factor, minimum_step;  // adaptive AP controller
    // With frame_end > 0 a launch walks order positions [frame_begin,
    // frame_end) of its one pass (one GD batch between regulariser steps),
    // adding its objective partials to the pass's when `accumulate`.
    int frame_begin, frame_end, accumulate;
    // Single-CTA engine: per-CTA field scratch, [launch CTAs][N * N], and
    // whether every tile has a unit pupil (TileDesc::pupil_span set).
    float2* field_scratch;
    int unit_pupils;
    // EPRY frame-gain and background recovery (src/algorithms/common.rs:390-489):
    // per-tile state (indexed like tiles), or null.
    const TileRecovery* recovery;
    int recover_gains, recover_background;
    double gain_step, gain_min, gain_max, background_step, background_min, background_max;
};

// Forward-model (simulate) parameters: one model, cluster per frame.
struct ForwardParams {
    const float2* object;      // M*M centred spectrum
    const float2* pupil;       // N*N
    const FrameParam* params;  // [frame_count]
    const float* background;   // natural layout, or null
    long long background_stride;
    float* out;                // frame_count * N*N natural-order intensities
    int M, frame_count;
};

bool engine_supported(int n);
// CTAs in the thread-block cluster that reconstructs one n x n tile.
int engine_ctas(int n);
// Field rows per CTA of an n x n tile (the stencil box is engine_rows(n) + 1 rows).
int engine_rows(int n);
// Stage-1 radix NA of the engine's row transform for an n x n tile: engine
// position t of a row holds natural column t / (n / NA) + NA * (t % (n / NA)),
// and engine row (y % C) * R + y / C holds natural row y.
int engine_na(int n);
// `clusters` clusters walk p.tile_count tiles (clusters <= p.tile_count).
cudaError_t launch_engine(int n, const EngineParams& p, int clusters, cudaStream_t s);
cudaError_t engine_max_active_clusters(int n, int* count);
cudaError_t launch_forward(int n, const ForwardParams& p, cudaStream_t s);

// Single-CTA frame engine (engine_l2.cu): one 512-thread CTA per tile, the
// field through a per-CTA scratch of engine_l2_scratch_bytes(n) bytes in
// p.field_scratch; 256-point tiles of the fixed-pupil projection families
// with amplitude-form measurements.
bool engine_l2_supported(int n, int alg);
size_t engine_l2_scratch_bytes(int n);
cudaError_t launch_engine_l2(int n, const EngineParams& p, int ctas, cudaStream_t s);
cudaError_t engine_l2_max_active_ctas(int n, int* count);

// Permutes natural-order frames [frames][N][N] into the engine layout.
cudaError_t launch_permute_f64_to_f32(int n, const double* src, float* dst, long long frames, cudaStream_t s);
cudaError_t launch_permute_u8(int n, const uint8_t* src, uint8_t* dst, long long frames, cudaStream_t s);
// Engine layout -> natural-order frames [frames][N][N], widened to FP64.
cudaError_t launch_unpermute_f32_to_f64(int n, const float* src, double* dst, long long frames, cudaStream_t s);

// Initial object (ReconstructionState::initialize_with_backend,
// src/reconstruction/state.rs:280-355) for a batch of tiles of one size:
// weighted mean amplitude -> nearest upsample into scratch (FP64).
struct InitTile {
    const float* meas;
    const uint8_t* masks;
    const float* background;
    long long background_stride;
    const FrameParam* params;
    double2* scratch;          // M*M natural-order FP64 object
    int* status;               // bit 2: no positive-weight unmasked pixel
    int frames_count;
    int amplitude;             // measurement form, as TileDesc::amplitude
};
// avg: [count * N*N] doubles; partial: [count * init_chunks(N) * 2] doubles.
int init_chunks(int n);
cudaError_t launch_init_mean(int n, int m, const InitTile* tiles, int count, double* avg, double* partial,
                             cudaStream_t s);

// FP64 mixed-radix line FFTs over a batch of arrays: lines of length n with
// element stride `stride` and line distance `dist`, `lines` lines per array.
cudaError_t launch_fft_lines(double2* const* arrays, int count, int n, long long stride, long long dist,
                             int lines, int inverse, const double2* roots, const int* factors, int nfactors,
                             double scale, cudaStream_t s);

// Centred float state <-> natural FP64 scratch conversions.
cudaError_t launch_shift_to_state(double2* const* scratch, float2* const* object, float2* const* anchor,
                                  float2* const* velocity, int count, int m, cudaStream_t s);
cudaError_t launch_state_to_natural(const float2* const* object, double2* const* scratch, int count, int m,
                                    cudaStream_t s);
// Detector response (CameraModel::measure_frame, src/simulation/camera.rs:249-290).
struct CameraParams {
    double photons_per_pixel, gain_counts_per_electron, offset_counts, read_noise, dark_current;
    double maximum_count;             // clamp; infinity when unbounded
    int shot_noise, quantize;
    const double* sensitivity;        // per-pixel sensitivity of one frame, or null
    unsigned long long seed;
};
// counts[e] from intensity[e] for e < total (frames of frame_len pixels).
// status bit 1: a Poisson draw hit its iteration bound.
cudaError_t launch_camera(const float* intensity, double* counts, long long total, long long frame_len,
                          const CameraParams& params, int* status, cudaStream_t s);

// Dense complex128 rows narrowed to complex64 rows of stride dst_stride.
cudaError_t launch_narrow(const double2* src, int rows, int cols, float2* dst, long long dst_stride, cudaStream_t s);
// Complex64 rows (row stride src_stride) widened to dense complex128.
cudaError_t launch_widen(const float2* src, long long src_stride, int rows, int cols, double2* dst, cudaStream_t s);

// Object/pupil gauge canonicalisation (src/algorithms/gauge.rs:20-73), one
// block per tile, FP64 reductions.
struct GaugeTile {
    float2* object;
    float2* pupil;
    const double2* reference;  // compiled pupil, FP64
    const uint8_t* support;
    int* status;               // bit 3: gauge failure
    int row_exact, col_exact;  // every source offset is integer on that axis
};
cudaError_t launch_gauge(const GaugeTile* tiles, int count, int n, int m, cudaStream_t s);

// GD regularisers between per-batch engine launches (src/algorithms/
// regularization.rs:5-80), FP64. Object TV: dst = src - weight * grad TV_eps
// on natural-order M x M objects. Pupil smoothing: dst = pupil - weight *
// grad |D pupil|^2 on the N x N state pupil, then the support when
// `constrain`; status bit 128 marks a non-finite result.
struct RegularTile {
    const double2* src;
    double2* dst;
    float2* pupil;
    float2* pupil_scratch;
    const uint8_t* support;
    double weight;
    int* status;
};
cudaError_t launch_object_tv(const RegularTile* tiles, int count, int m, double epsilon, cudaStream_t s);
cudaError_t launch_pupil_smoothing(const RegularTile* tiles, int count, int n, int constrain, cudaStream_t s);

// GD illumination recovery (src/algorithms/gradient_descent.rs:1044-1089,
// 1236-1368). Per tile: the run's own copy of the frame constants, whose
// stencil fields follow the recovered offsets, the compiled crop starts and
// offsets, and the (row, column) corrections in FP64.
struct IlluminationTile {
    const float2* object;      // M x (M + M % 2) centred spectrum (state)
    const float2* pupil;       // N*N centred state pupil
    const float* meas;         // engine layout, as TileDesc::meas
    const uint8_t* masks;      // engine layout, or null
    const float* background;   // engine layout, or null
    long long background_stride;
    FrameParam* params;        // [frame_count], rewritten by the update
    const int* order;          // [frame_count] schedule, or null
    const long long* start;    // [frame_count][2] crop start (row, column)
    const double* offset;      // [frame_count][2] compiled subpixel offset
    double* correction;        // [frame_count][2] recovered correction
    double* partials;          // [frame_count][kIlluminationBlocks][4] (gradient row, column, curvature row, column)
    int* status;               // bit 256: non-finite illumination gradient or curvature
    int M, frame_count, amplitude;
};
// Pixel slices (blocks) per task of the finite-difference reduction; the
// update sums their partials in a fixed order.
constexpr int kIlluminationBlocks = 32;
// One gradient evaluation: order position `position` of tile `tile`.
struct IlluminationTask {
    int tile, position;
};
// Finite differences of one chunk of tasks in FP64: per task five N x N
// fields (the current offset, then +-d on rows and on columns), each the
// ifftshifted patch x pupil before and the detector field after the
// inverse FFT; `valid` flags the evaluations whose stencil is inside the grid.
struct IlluminationParams {
    const IlluminationTile* tiles;
    const IlluminationTask* tasks;
    double2* fields;           // [tasks][5][N*N]
    int* valid;                // [tasks][5]
    double distance, epsilon;
    int loss, n;
};
cudaError_t launch_illumination_fields(const IlluminationParams& p, int tasks, cudaStream_t s);
cudaError_t launch_illumination_reduce(const IlluminationParams& p, int tasks, cudaStream_t s);
cudaError_t launch_illumination_update(const IlluminationTile* tiles, const IlluminationTask* tasks, int count,
                                       int n, double step, double bound, double epsilon, cudaStream_t s);

// One axis of interpolation_axis (src/model/crop.rs:266-313) in FP64: the
// lower start and the upper fraction; false when the stencil leaves [0, m).
__host__ __device__ inline bool offset_axis(long long start, int n, int m, double offset, long long& lower,
                                            double& fraction) {
    if (!(fabs(offset) <= 1.7976931348623157e308)) return false;
    const double nearest = round(offset);
    double integer_offset;
    if (fabs(offset - nearest) <= 1e-12) {
        integer_offset = nearest;
        fraction = 0.0;
    } else {
        integer_offset = floor(offset);
        fraction = offset - integer_offset;
    }
    lower = start + (long long)integer_offset;
    const long long end = lower + n;
    return lower >= 0 && end <= m && !(fraction > 0.0 && end >= m);
}

// Stencil of a crop at a subpixel offset (CropIndices::validate_subpixel_inside
// and interpolation_axis, src/model/crop.rs:105-113, 266-313), the same
// arithmetic as the host's frame constants; false when it leaves the M x M
// grid. Keeps the frame's weight, gain and scale fields.
__host__ __device__ inline bool offset_frame_param(long long start_row, long long start_col, double off_row,
                                                   double off_col, int n, int m, FrameParam& fp) {
    long long lr, lc;
    double fr, fc;
    if (!offset_axis(start_row, n, m, off_row, lr, fr) || !offset_axis(start_col, n, m, off_col, lc, fc)) return false;
    if (fabs(off_row) <= 1e-12 && fabs(off_col) <= 1e-12) {
        fp.lower_row = (int)start_row;
        fp.lower_col = (int)start_col;
        fp.has_upper_row = fp.has_upper_col = 0;
        fp.w00 = 1.f;
        fp.w01 = fp.w10 = fp.w11 = 0.f;
        return true;
    }
    fp.lower_row = (int)lr;
    fp.lower_col = (int)lc;
    fp.has_upper_row = fr > 0.0 ? 1 : 0;
    fp.has_upper_col = fc > 0.0 ? 1 : 0;
    fp.w00 = (float)((1.0 - fr) * (1.0 - fc));
    fp.w01 = (float)((1.0 - fr) * fc);
    fp.w10 = (float)(fr * (1.0 - fc));
    fp.w11 = (float)(fr * fc);
    return true;
}

// Context accessors for entry points that live outside runtime.cpp.
void set_context_error(fpm_context* ctx, const char* message);
void context_device_stream(fpm_context* ctx, int* device, cudaStream_t* stream);
// The context's own lock, held by every entry point that uses its streams or error text.
std::mutex& context_mutex(fpm_context* ctx);

}  // namespace fpm
