/*
 * fpm_gpu.h - C ABI of the GB300 (sm_103a) device backend for fpm-rs's
 * image-plane FPM forward model and reconstruction inner loop.
 *
 * All entry points are extern "C", take plain pointers and sizes, and return an
 * int32_t status (FPM_OK on success). Host arrays are caller-owned, row-major
 * and C-contiguous, and are only read (or written, for outputs) for the
 * duration of the call. Complex arrays are interleaved (re, im) float64, the
 * layout of Rust's Complex64 and NumPy's complex128. Device buffers are owned
 * by opaque handles; no device pointer crosses the boundary.
 *
 * Replaced reference interfaces (paths are within hgrecco/fpm-rs):
 *   Backend::fft2 ................ src/backend/traits.rs:123-131 -> fpm_fft2
 *   ImagePlaneModel::compile ..... src/model/image_plane_fpm.rs:196-253 -> fpm_compile_model
 *   ForwardModel::forward_intensity_stack_into
 *                                  src/model/forward.rs:300-372 -> fpm_forward_stack
 *   Simulator::simulate + CameraModel::measure_frame
 *                                  src/simulation/simulator.rs:107-206, camera.rs:249-290 -> fpm_simulate_stack
 *   ReconstructionProblem::new ... src/reconstruction/problem.rs:12-20 -> fpm_problem_create,
 *                                  fpm_problem_create_batch (many problems, one host scan)
 *   Runner::run / ReconstructionAlgorithm::run
 *                                  src/reconstruction/runner.rs:76-285 -> fpm_run
 *   AdaptiveAlternatingProjection  src/algorithms/adaptive_alternating_projection.rs:245-470
 *                                  -> fpm_run with FPM_ALG_ADAPTIVE_AP
 *   ReconstructionCheckpoint capture / run_from_checkpoint
 *                                  src/reconstruction/checkpoint.rs:38-146 -> fpm_run_batch_resumable
 *   SpectralRunner::run + SpectralAlternatingProjection
 *                                  src/reconstruction/spectral.rs:494-642,
 *                                  src/algorithms/spectral.rs:182-271 -> fpm_spectral_run,
 *                                  fpm_spectral_run_batch (many requests, one launch per tile size)
 *   SpectralImagePlaneModel::forward_intensity
 *                                  src/model/spectral.rs:400-446 -> fpm_spectral_forward
 *   (new) serving ................ fpm_run_batch_submit + fpm_job_poll / fpm_job_wait
 *   (new) batched tiles .......... fpm_run_batch (many independent problems, one launch per tile size),
 *                                  fpm_run_batch_host (host inputs, copies overlapped with the runs)
 *   Error / FpmError ............. src/error.rs:12, python/src/errors.rs:17-50 -> FPM_ERR_* + fpm_last_error
 */
#ifndef FPM_GPU_H
#define FPM_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes, one per reference Error variant that this path can raise. */
enum {
    FPM_OK = 0,
    FPM_ERR_INVALID_SHAPE = 1,        /* Error::InvalidShape */
    FPM_ERR_INVALID_PARAMETER = 2,    /* Error::InvalidParameter */
    FPM_ERR_INVALID_MODEL = 3,        /* Error::InvalidModel */
    FPM_ERR_INVALID_MEASUREMENTS = 4, /* Error::InvalidMeasurements */
    FPM_ERR_LENGTH_MISMATCH = 5,      /* Error::LengthMismatch */
    FPM_ERR_FRAME_OUT_OF_RANGE = 6,   /* Error::FrameOutOfRange */
    FPM_ERR_NUMERICAL = 7,            /* Error::Numerical */
    FPM_ERR_UNSUPPORTED = 8,          /* Error::Unsupported */
    FPM_ERR_CUDA = 9,                 /* a CUDA runtime call failed */
    FPM_ERR_TIMEOUT = 10,             /* a bounded device wait expired (frame-engine stencil load) */
    FPM_ERR_QUEUE_FULL = 11           /* serving: the server's queue is full, the request was not taken */
};

enum { FPM_SHAPE_EXACT = 0, FPM_SHAPE_MINIMUM = 1, FPM_SHAPE_SMOOTH = 2, FPM_SHAPE_POWER_OF_TWO = 3 };
enum { FPM_LOSS_AMPLITUDE_MSE = 0, FPM_LOSS_INTENSITY_MSE = 1, FPM_LOSS_POISSON_NLL = 2, FPM_LOSS_HUBER_AMPLITUDE = 3 };
enum { FPM_ALG_AP = 0, FPM_ALG_FPIE = 1, FPM_ALG_MPIE = 2, FPM_ALG_EPRY = 3, FPM_ALG_GD = 4, FPM_ALG_ADAPTIVE_AP = 5 };
enum {
    FPM_SCHEDULE_SEQUENTIAL = 0,
    FPM_SCHEDULE_BRIGHTFIELD_FIRST = 1,
    FPM_SCHEDULE_SPIRAL_OUT = 2,
    FPM_SCHEDULE_SNR_WEIGHTED = 3
};

typedef struct fpm_context fpm_context;
typedef struct fpm_problem fpm_problem;
typedef struct fpm_job fpm_job;
typedef struct fpm_plan fpm_plan;
typedef struct fpm_server fpm_server;

/* Microscope optics (src/experiment/optics.rs:44-68). */
typedef struct {
    double wavelength_vacuum_m, objective_na, magnification, camera_pixel_size;
    double illumination_refractive_index, objective_medium_refractive_index;
    int32_t has_defocus;
    double defocus_distance;
    int32_t has_aberration;
    double astigmatism, coma, spherical, edge_apodization;
} fpm_optics;

/* Compiled, non-multiplexed image-plane model (src/model/image_plane_fpm.rs:57-73).
 * frames == sources. Offsets may be NULL (integer crops). */
typedef struct {
    int32_t image_height, image_width;
    int32_t recon_height, recon_width;
    int32_t sources;
    const int64_t *crop_start_row, *crop_start_col; /* [sources] */
    const double *offset_row, *offset_col;          /* [sources] or NULL */
    const double *pupil;                            /* complex128 [h*w] */
    const uint8_t *support;                         /* [h*w], 0 or 1 */
    const double *frame_gains;                      /* [sources] or NULL (all 1) */
    const double *background;                       /* NULL, [h*w] or [sources*h*w] */
    int64_t background_len;
    const double *kx, *ky;                          /* [sources] rad/m; used by sorted schedules */
} fpm_model_desc;

/* Measurement stack (src/measurements/stack.rs:47-...). */
typedef struct {
    int32_t frames;
    const double *measurements;  /* [frames*h*w] float64 */
    const double *frame_weights; /* [frames] or NULL (all 1) */
    const uint8_t *masks;        /* [frames*h*w] or NULL; 0 excludes a pixel */
} fpm_measurement_desc;

/* Algorithm parameters; fields not used by an algorithm are ignored.
 * Defaults: AlternatingProjection src/algorithms/alternating_projection.rs:51-61,
 * Fpie src/algorithms/fpie.rs, Mpie src/algorithms/mpie.rs:81-95,
 * Epry src/algorithms/epry.rs:91-112, GradientDescent
 * src/algorithms/gradient_descent.rs:171-193. */
typedef struct {
    int32_t algorithm;
    int32_t iterations;
    int32_t batch_size;
    int32_t loss_type;
    int32_t schedule;
    double object_step;
    double epsilon;
    double stability;            /* FPIE / mPIE */
    int32_t momentum_interval;   /* mPIE */
    double momentum_friction;    /* mPIE */
    double momentum_feedback;    /* mPIE */
    int32_t recover_pupil;       /* EPRY */
    int32_t constrain_pupil_support;
    double pupil_step;
    int32_t recover_frame_gains; /* EPRY: per-frame gain recovery (gain_step, gain_min, gain_max below) */
    int32_t recover_background;  /* EPRY: per-frame background recovery (background_step, _min, _max below) */
    int32_t poisson_truncation;  /* GD: nonzero enables the Poisson truncation gate */
    double poisson_truncation_threshold; /* GD: the gate's threshold (finite, positive; Poisson NLL only) */
    /* Adaptive AP (object_step is the initial step): the step is multiplied by
     * reduction_factor, not below minimum_object_step, after a pass whose
     * relative objective progress is at most progress_threshold. */
    double progress_threshold, reduction_factor, minimum_object_step;
    /* GD regularisers at every batch end, scaled by the batch's share of the
     * frames (src/algorithms/gradient_descent.rs:643-660): an isotropic TV
     * step on the real-space object (weight 0: off; epsilon finite and > 0
     * when on) and, with pupil recovery, a quadratic smoothing step on the
     * pupil before its support is imposed. */
    double object_tv_weight, object_tv_epsilon, pupil_smoothing_weight;
    /* GD illumination recovery (GradientDescent::recover_illumination,
     * src/algorithms/gradient_descent.rs:146-153, 1044-1089, 1236-1368): per
     * source, a Gauss-Newton step of illumination_step on finite differences
     * at +-illumination_finite_difference subpixels, clamped to
     * +-maximum_illumination_correction and kept only while the corrected crop
     * stays inside the grid. The three values are validated (finite and
     * positive) when recover_illumination is set. Not combined with pupil
     * recovery, Poisson truncation or resumed runs on the device path. */
    int32_t recover_illumination;
    double illumination_step, illumination_finite_difference, maximum_illumination_correction;
    /* Compensated (Kahan) summation of the per-frame updates into the
     * complex64 object spectrum, or into the mini-batch gradient: each grid
     * cell carries its rounding error, folded back at the end of every
     * launch. Costs one more complex64 read and write per stencil cell. 0:
     * plain FP32 accumulation. */
    int32_t compensated_accumulation;
    /* EPRY frame-gain and background recovery (update_gain and
     * update_background, src/algorithms/common.rs:390-489; Epry::validate,
     * src/algorithms/epry.rs:206-236). Each frame's gain moves by gain_step
     * toward sum p (y - b)+ / sum p^2 (clamped to [gain_min, gain_max]), then
     * its background by background_step times the mean residual y - g p - b
     * (clamped to [background_min, background_max]), before the projection
     * uses them. Steps in [0, 1]; gain bounds finite, positive, increasing;
     * background bounds finite, increasing. Validated only when the matching
     * recovery is set; not combined with resumed runs. Amplitude-form
     * problems (no model background) read their intensities as g0 a^2 from
     * the stored a = sqrt(max(y / g0, 0)). */
    double gain_step, gain_min, gain_max;
    double background_step, background_min, background_max;
} fpm_algorithm_params;

/* Result buffers; any pointer may be NULL. */
typedef struct {
    double *object;          /* complex128 [mh*mw] real-space object */
    double *object_spectrum; /* complex128 [mh*mw] centred spectrum */
    double *pupil;           /* complex128 [h*w] recovered pupil */
    double *objectives;      /* [iterations] weighted mean objective per iteration */
    int32_t completed_iterations;
    /* [sources*2] recovered (row, column) illumination corrections
     * (ReconstructionResult::calibrated_illumination, src/reconstruction/
     * result.rs:94); written only by runs with recover_illumination. */
    double *illumination_corrections;
    /* EPRY runs that recover them: [sources] frame gains and
     * [sources*h*w] backgrounds (ReconstructionResult::recovered_frame_gains
     * and recovered_background). */
    double *frame_gains;
    double *background;
} fpm_result_desc;

/* ------------------------------------------------------------------ context */
int32_t fpm_create(fpm_context **ctx, int32_t device);
/* Problems, jobs and plans refer to their context: destroy them (waiting for
 * jobs) before the context. */
int32_t fpm_destroy(fpm_context *ctx);
/* Copies the last error message of this context (NUL-terminated, truncated). */
int32_t fpm_last_error(const fpm_context *ctx, char *buffer, size_t length);
/* Library-wide last error, for failures before a context exists. */
const char *fpm_global_last_error(void);

/* --------------------------------------------------------- host geometry */
/* Planar LED array k-vectors (src/experiment/led_array.rs:292-313 and
 * src/experiment/illumination.rs:385-421). translation/rotation are [3]. */
int32_t fpm_planar_led_kvectors(const fpm_optics *optics, int32_t rows, int32_t cols, double pitch_x,
                                double pitch_y, double reference_col, double reference_row,
                                const double *translation, const double *rotation_rad, double *kx,
                                double *ky);
/* Resolves the reconstruction shape only (suggest_reconstruction_shape). */
int32_t fpm_suggest_shape(const fpm_optics *optics, int32_t sources, const double *kx, const double *ky,
                          int32_t image_height, int32_t image_width, int32_t policy, int32_t *recon_height,
                          int32_t *recon_width);
/* Mean loss (FPM_LOSS_*) between count > 0 finite predicted and measured
 * intensities, summed in order in FP64 on the host: the objective's data term
 * (src/algorithms/objective.rs:27-72), which the Python binding exposes as
 * intensity_loss (python/src/metrics.rs:248-269). */
int32_t fpm_intensity_loss(const double *predicted, const double *measured, int64_t count, int32_t loss_type,
                           double *out);
/* Compiles k-vectors into crops, fractional offsets and the circular pupil.
 * Caller allocates start_row/start_col/offset_row/offset_col [sources],
 * pupil [2*h*w] and support [h*w]. For FPM_SHAPE_EXACT the shape is read from
 * the values recon_height and recon_width point to; otherwise it is written there. */
int32_t fpm_compile_model(const fpm_optics *optics, int32_t sources, const double *kx, const double *ky,
                          int32_t image_height, int32_t image_width, int32_t policy, int32_t *recon_height,
                          int32_t *recon_width, int64_t *start_row, int64_t *start_col, double *offset_row,
                          double *offset_col, double *pupil, uint8_t *support, double *dkx, double *dky);

/* ------------------------------------------------------------- device work */
/* Backend::fft2 on host data: complex128 [h*w] in place, reference convention
 * (forward scaled by 1/(h*w), inverse unscaled). Computed in FP64 on the GPU. */
int32_t fpm_fft2(fpm_context *ctx, double *values, int32_t height, int32_t width, int32_t inverse);

/* fpm_fft2 without device allocation, for callers that cannot call
 * cudaMalloc (device memory owned by another allocator or admitted against a
 * fixed HBM budget; loops that must not synchronise the device). No
 * counterpart in the reference. Scratch is one fixed file-scope device array
 * (768*768 complex128 values, at most 4096 per row or column; larger shapes
 * return FPM_ERR_INVALID_SHAPE) that each GPU holds until the process exits.
 * Calls are serialised by a process-wide lock because they share that array.
 * The first call on a device looks up the array's address; make it before any
 * stream capture. That first call (or the module load, where modules load
 * eagerly) also commits the array's 9 MiB on the device: callers that budget
 * device memory should make one call during their set-up. */
int32_t fpm_fft2_noalloc(fpm_context *ctx, double *values, int32_t height, int32_t width, int32_t inverse);

/* Forward intensity stack [sources*h*w] of a complex128 object [mh*mw]
 * (object FFT, crop, pupil, IFFT, |psi|^2 * gain + background). */
int32_t fpm_forward_stack(fpm_context *ctx, const fpm_model_desc *model, const double *object,
                          double *intensities);

/* Detector response of CameraModel (src/simulation/camera.rs:249-318). */
typedef struct {
    double photons_per_pixel;        /* expected electrons = max(I, 0) * sensitivity * photons + dark */
    double gain_counts_per_electron;
    double offset_counts;
    double read_noise_electrons;     /* standard deviation of Gaussian read noise, 0 for none */
    double dark_current_electrons;
    int32_t shot_noise;              /* Poisson electrons */
    int32_t quantize;                /* round counts (half away from zero) */
    double maximum_count;            /* counts are clamped to [0, maximum_count]; INFINITY for none */
    const double *pixel_sensitivity; /* h*w, or NULL */
    const int64_t *bad_pixels;       /* pixel indices within a frame, or NULL */
    int64_t bad_pixel_count;
    double bad_pixel_value;          /* counts of a bad pixel; NAN for maximum_count */
} fpm_camera_desc;

/* Simulator::simulate's measurement stack (src/simulation/simulator.rs:
 * 107-206) on the device: the forward intensity stack of `object`, then the
 * detector, counts[sources*h*w]. Random draws come from a counter-based
 * generator keyed by `seed` (reproducible for a given seed; equal to the
 * reference's ChaCha12 draws only in distribution). */
int32_t fpm_simulate_stack(fpm_context *ctx, const fpm_model_desc *model, const double *object,
                           const fpm_camera_desc *camera, uint64_t seed, double *counts);

/* Uploads a validated model + measurement pair; the problem keeps its
 * measurements resident on the device until fpm_problem_destroy. */
int32_t fpm_problem_create(fpm_context *ctx, const fpm_model_desc *model,
                           const fpm_measurement_desc *measurements, fpm_problem **problem);
int32_t fpm_problem_destroy(fpm_problem *problem);

/* Creates `count` problems from parallel arrays of descriptors, as
 * fpm_problem_create would one by one: every frame of every problem is
 * validated in one pass over the host's threads, then all uploads run with a
 * single final synchronisation. On error no problem is returned (all entries
 * of `problems` are set to NULL) and the message names the failing index. */
int32_t fpm_problem_create_batch(fpm_context *ctx, int32_t count, const fpm_model_desc *models,
                                 const fpm_measurement_desc *measurements, fpm_problem **problems);

/* Runs one reconstruction to completion (initialise, iterate, finalise). */
int32_t fpm_run(fpm_context *ctx, fpm_problem *problem, const fpm_algorithm_params *params,
                fpm_result_desc *result);

/* Runs `count` independent reconstructions with the same parameters. Tiles of
 * one image size share a launch; sizes run concurrently on separate streams.
 * Each tile keeps the exact sequential frame order of a single run. */
int32_t fpm_run_batch(fpm_context *ctx, int32_t count, fpm_problem *const *problems,
                      const fpm_algorithm_params *params, fpm_result_desc *results);

/* Resumable reconstruction state, the device counterpart of
 * ReconstructionCheckpoint (src/reconstruction/checkpoint.rs:38-52):
 * complex128 arrays, centred object spectrum. As an input it restores a run;
 * as an output the library fills the caller's arrays. The device state is
 * complex64, so a capture restores exactly and a resumed run reproduces the
 * uninterrupted one bit for bit. */
typedef struct {
    int32_t completed_iterations;   /* complete iterations the state represents */
    int32_t momentum_counter;       /* mPIE: effective frames since the last momentum event */
    double *object_spectrum;        /* mh*mw complex */
    double *pupil;                  /* h*w complex */
    double *velocity;               /* mPIE: mh*mw complex, else NULL */
    double *anchor;                 /* mPIE: mh*mw complex, else NULL */
    double *objectives;             /* one objective per completed iteration (the trace) */
    /* GD illumination recovery: sources*2 (row, column) corrections
     * (ReconstructionCheckpoint::illumination_corrections, src/reconstruction/
     * checkpoint.rs:44), or NULL (none recovered yet: zeros on resume). */
    double *illumination_corrections;
} fpm_state_desc;

/* fpm_run_batch that can start from saved state and save state at the end.
 * `resume` (count entries, or NULL) restores each problem's state and runs
 * iterations [completed_iterations, params->iterations); every entry must
 * have the same completed_iterations. Results carry the full objective
 * trace, resumed prefix included. `capture` (count entries, or NULL)
 * receives each problem's state after the run; its objectives array holds
 * params->iterations values. */
int32_t fpm_run_batch_resumable(fpm_context *ctx, int32_t count, fpm_problem *const *problems,
                                const fpm_algorithm_params *params, const fpm_state_desc *resume,
                                fpm_result_desc *results, fpm_state_desc *capture);

/* fpm_problem_create_batch + fpm_run_batch for host-resident inputs, with
 * the copies overlapped: problems are created, run and downloaded in chunks
 * (largest tiles first, at most 2 GiB of float64 measurements each), so the
 * validation and upload of one chunk run beside the reconstruction of the
 * previous ones and downloads overlap the runs still in flight. Results are
 * identical to the two-call form. The created problems are returned in
 * `problems` (caller-owned, resident for later runs; fpm_problem_destroy
 * frees them); on error none is returned. */
int32_t fpm_run_batch_host(fpm_context *ctx, int32_t count, const fpm_model_desc *models,
                           const fpm_measurement_desc *measurements, const fpm_algorithm_params *params,
                           fpm_result_desc *results, fpm_problem **problems);

/* Device-side statistics of the last fpm_run / fpm_run_batch, from CUDA
 * events recorded on the streams the kernels ran on. */
typedef struct {
    int32_t kernel_launches;   /* every kernel this library launched */
    int32_t engine_launches;   /* frame-engine launches */
    double run_ms;             /* first kernel start to last kernel end */
    double engine_ms_sum;      /* sum of frame-engine launch durations */
    double engine_span_ms;     /* first engine start to last engine end */
    double engine_bytes;       /* algorithmic HBM bytes of the engine launches */
    int32_t buckets;           /* tile-size groups of the run (at most 8 reported) */
    int32_t bucket_size[8];    /* detector size N of each group */
    int32_t bucket_tiles[8];   /* tiles in each group */
    double bucket_end_ms[8];   /* run start to the group's results being ready */
    /* fpm_run_batch_host only (0 otherwise), host wall times in ms from the
     * call's start: until the first chunk's device work was queued, spent
     * validating measurements, spent in measurement uploads, and the whole
     * call. */
    double host_first_launch_ms, host_scan_ms, host_upload_ms, host_call_ms;
    /* fpm_run_batch_host only: the call's chunks (at most 16 reported), each
     * with its tile count and the time its results were on the host. */
    int32_t host_chunks;
    int32_t host_done_tiles[16];
    double host_done_ms[16];
} fpm_run_stats;

int32_t fpm_last_run_stats(const fpm_context *ctx, fpm_run_stats *stats);


/* ------------------------------------------------- narrowband spectral AP */
/* ObjectCoupling (src/model/spectral.rs:21-30). */
enum { FPM_COUPLING_INDEPENDENT = 0, FPM_COUPLING_SHARED_COMPLEX = 1 };

/* SpectralImagePlaneModel (src/model/spectral.rs:46-54): channel kernels
 * compiled on one common grid (equal image and reconstruction shapes, no
 * background) and the canonical sparse detector plan
 * (SpectralAcquisitionPlan, src/experiment/spectral.rs:44-70). Exposure e
 * sums contributions [contribution_offsets[e], contribution_offsets[e + 1]):
 * (channel, local frame, spectral weight > 0), unique per exposure. */
typedef struct {
    int32_t channels;
    const fpm_model_desc *channel_models;   /* [channels] */
    int32_t object_coupling;                /* FPM_COUPLING_* */
    int32_t exposures;                      /* physical detector frames */
    const int32_t *contribution_offsets;    /* [exposures + 1], starting at 0 */
    const int32_t *contribution_channel;    /* [contributions] */
    const int32_t *contribution_local_frame;
    const double *contribution_weight;
    const double *exposure_gain;            /* [exposures], finite and > 0 */
    const double *exposure_background;      /* [exposures], finite and >= 0 */
} fpm_spectral_model_desc;

/* SpectralAlternatingProjection (src/algorithms/spectral.rs:111-145);
 * defaults iterations 50, batch_size 1, amplitude MSE, object_step 1,
 * epsilon 1e-10. batch_size does not change the per-exposure updates. */
typedef struct {
    int32_t iterations;
    int32_t batch_size;
    int32_t loss_type;      /* diagnostic objective, FPM_LOSS_* */
    double object_step;
    double epsilon;
} fpm_spectral_params;

/* Object-only spectral alternating projection on the device. Stored objects:
 * one per channel (independent) or one (shared complex), each mh*mw.
 *   order            NULL (acquisition order) or a permutation of the exposures, every pass
 *   initial_objects  NULL (measured-amplitude initialisation) or natural-order complex objects
 *   resume_spectra   NULL, or centred spectra after completed_iterations passes (a checkpoint)
 * Outputs, each NULL or sized for the stored objects: objects (natural order),
 * object_spectra (centred), objectives [iterations - completed_iterations],
 * the weighted mean diagnostic loss of each pass before its updates. */
int32_t fpm_spectral_run(fpm_context *ctx, const fpm_spectral_model_desc *model,
                         const fpm_measurement_desc *measurements, const fpm_spectral_params *params,
                         const int32_t *order, const double *initial_objects, const double *resume_spectra,
                         int32_t completed_iterations, double *objects, double *object_spectra,
                         double *objectives);

/* Result buffers of one spectral problem; any pointer may be NULL. */
typedef struct {
    double *objects;         /* object_count*mh*mw complex, natural order */
    double *object_spectra;  /* object_count*mh*mw complex, centred */
    double *objectives;      /* [iterations] */
} fpm_spectral_result_desc;

/* fpm_spectral_run for `count` independent problems (acquisition order,
 * measured-amplitude initialisation) with one engine launch per tile size:
 * each problem is one thread-block cluster, so a batch of requests fills the
 * GPU where one request occupies a single cluster. Results equal separate
 * fpm_spectral_run calls. */
int32_t fpm_spectral_run_batch(fpm_context *ctx, int32_t count, const fpm_spectral_model_desc *models,
                               const fpm_measurement_desc *measurements, const fpm_spectral_params *params,
                               fpm_spectral_result_desc *results);

/* Detector intensities of every exposure, [exposures*h*w], from the stored
 * objects' centred spectra: gain * sum(weight * local intensity) + background. */
int32_t fpm_spectral_forward(fpm_context *ctx, const fpm_spectral_model_desc *model, const double *spectra,
                             double *intensities);

/* ------------------------------------------------------------ serving */
/* fpm_run_batch without the wait, for serving loops: the work is queued on
 * the job's own streams (jobs of one context overlap) and the call returns.
 * Until the job has finished, its problems are reserved (other calls and
 * fpm_problem_destroy refuse them) and `results` and its arrays must stay
 * valid; `params` is copied. */
int32_t fpm_run_batch_submit(fpm_context *ctx, int32_t count, fpm_problem *const *problems,
                             const fpm_algorithm_params *params, fpm_result_desc *results, fpm_job **job);
/* fpm_spectral_run_batch without the wait: measurement uploads and the
 * initial objects are queued before the call returns, so the descriptors
 * and their arrays need to outlive the call only; `results` must stay valid
 * until the job has finished. */
int32_t fpm_spectral_run_batch_submit(fpm_context *ctx, int32_t count, const fpm_spectral_model_desc *models,
                                      const fpm_measurement_desc *measurements, const fpm_spectral_params *params,
                                      fpm_spectral_result_desc *results, fpm_job **job);
/* Non-blocking: *done = 1 once the device work has finished; the call that
 * first sees it downloads the results (a short wait on the finished work)
 * and fills the objectives, then returns the job's status. */
int32_t fpm_job_poll(fpm_job *job, int32_t *done);
/* Blocks until the job has finished; returns its status. */
int32_t fpm_job_wait(fpm_job *job);
/* Device statistics of a finished job (as fpm_last_run_stats). */
int32_t fpm_job_stats(fpm_job *job, fpm_run_stats *stats);
/* Waits for the job if needed and frees it. */
int32_t fpm_job_destroy(fpm_job *job);

/* ----------------------------------------------------- captured run plans */
/* Runner::run over a batch (src/reconstruction/runner.rs:76-285) recorded
 * once as a CUDA graph: the device work of fpm_run_batch for these problems
 * and parameters (initialisation, frame engine, per-iteration gauge,
 * regulariser and illumination steps, finalisation; every tile size on its
 * own stream) becomes one graph launch. Each replay starts from the problems'
 * initial state, exactly as a fresh fpm_run_batch, and leaves its results on
 * the device. The problems are held by the plan until fpm_plan_destroy
 * (other runs and fpm_problem_destroy refuse them); resumed runs are not
 * captured. */
int32_t fpm_plan_create(fpm_context *ctx, int32_t count, fpm_problem *const *problems,
                        const fpm_algorithm_params *params, fpm_plan **plan);
/* Queues one replay on the context's first stream and returns. */
int32_t fpm_plan_launch(fpm_plan *plan);
/* Waits for the replays queued so far, checks every problem's device status
 * and records the last replay's statistics (fpm_last_run_stats). */
int32_t fpm_plan_wait(fpm_plan *plan);
/* Downloads the last replay's results, as fpm_run_batch fills `results`
 * (indexed like the plan's problems). */
int32_t fpm_plan_collect(fpm_plan *plan, fpm_result_desc *results);
/* Waits for queued replays and frees the plan; its problems are free again. */
int32_t fpm_plan_destroy(fpm_plan *plan);

/* -------------------------------------------------- frame-engine launches */
/* A frame-engine launch of one tile size runs `clusters` thread-block
 * clusters that walk the launch's tiles (cluster k takes tiles k, k + G, ...);
 * 0 (the default) gives every tile its own cluster. Autotuners set it per
 * tile size n in {32, 64, 128, 256}. */
int32_t fpm_set_engine_grid(fpm_context *ctx, int32_t n, int32_t clusters);
/* Clusters of an n x n tile's frame engine that fit on the device at once
 * (CTAs when the tile size's shape is FPM_ENGINE_SINGLE_CTA or _AUTO). */
int32_t fpm_engine_max_clusters(fpm_context *ctx, int32_t n, int32_t *clusters);
/* Frame-engine shape of a tile size. FPM_ENGINE_CLUSTER splits a tile over
 * a thread-block cluster (rows across CTAs, exchanges through distributed
 * shared memory). FPM_ENGINE_SINGLE_CTA gives a tile one 512-thread CTA
 * whose 2-D transforms pass through a per-CTA field scratch held in L2
 * (256-point tiles of AP, FPIE, mPIE and EPRY without pupil recovery, with
 * measurements that have no background and plain accumulation; other runs
 * keep the cluster engine): a higher throughput over many tiles, a longer
 * time for one. FPM_ENGINE_AUTO takes the single-CTA engine for launches of
 * at least two thirds of the CTAs that fit at once, else the cluster
 * engine. Default: AUTO for n = 256, the cluster engine for the other
 * sizes. Both shapes compute the update of src/algorithms/common.rs:57-306
 * with the same arithmetic per value; fpm_set_engine_grid applies to
 * cluster launches, fpm_set_engine_ctas to single-CTA launches. */
enum { FPM_ENGINE_CLUSTER = 0, FPM_ENGINE_SINGLE_CTA = 1, FPM_ENGINE_AUTO = 2 };
int32_t fpm_set_engine_shape(fpm_context *ctx, int32_t n, int32_t shape);
/* CTAs of a single-CTA engine launch of tile size n, which walk the
 * launch's tiles as the clusters do (0, the default: as many as fit at once). */
int32_t fpm_set_engine_ctas(fpm_context *ctx, int32_t n, int32_t ctas);

/* ------------------------------------------------------- serving loop */
/* A request loop over one context: the work run_algorithm
 * (python/src/reconstruction.rs:1107-1141) does for one caller, served to
 * many with continuous batching. A dispatcher thread admits waiting
 * requests in arrival order while their device footprint fits the budget
 * beside the work in flight, sends requests of equal parameters that arrive
 * within the batching window as one submitted batch, and admits more as
 * batches finish, so new requests overlap the ones on the GPU. Each
 * result is the one a run of that request alone gives. */
typedef struct {
    int64_t hbm_budget_bytes; /* admitted requests' device footprint at most this; 0: no limit */
    int32_t max_batch;        /* requests of equal parameters per submitted batch, >= 1 */
    double batch_window_ms;   /* how long the oldest waiting request waits for batch-mates */
    int64_t max_queue;        /* waiting requests at most this (more get FPM_ERR_QUEUE_FULL); 0: no limit */
} fpm_server_config;

/* One request's times (host clock, ms since the server's creation),
 * footprint and outcome. */
typedef struct {
    double submit_ms, admit_ms, start_ms, done_ms;
    int64_t footprint_bytes;
    int32_t status;
    char message[256];
} fpm_request_info;

typedef struct {
    int64_t submitted, admitted, completed, rejected, batches;
    int64_t in_use_bytes, peak_bytes, waiting, in_flight_batches;
} fpm_server_stats;

int32_t fpm_server_create(fpm_context *ctx, const fpm_server_config *config, fpm_server **server);
/* Queues one request and returns its id. The descriptors are copied; the
 * arrays they point to (inputs and the result arrays) must stay valid until
 * fpm_server_wait returns for this request. */
int32_t fpm_server_submit(fpm_server *server, const fpm_model_desc *model, const fpm_measurement_desc *measurements,
                          const fpm_algorithm_params *params, fpm_result_desc *result, uint64_t *request);
/* Non-blocking: *done = 1 once the request's results are in its arrays. */
int32_t fpm_server_poll(fpm_server *server, uint64_t request, int32_t *done);
/* Blocks until the request has finished, fills `info` (may be NULL), forgets
 * the request and returns its status. */
int32_t fpm_server_wait(fpm_server *server, uint64_t request, fpm_request_info *info);
int32_t fpm_server_stats_get(fpm_server *server, fpm_server_stats *stats);
/* Finishes every queued and running request, then stops the dispatcher. */
int32_t fpm_server_destroy(fpm_server *server);

#ifdef __cplusplus
}
#endif

#endif
