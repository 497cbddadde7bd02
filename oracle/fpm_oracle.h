/*
 * FP64 CPU oracle for the fpm-rs image-plane FPM hot path.
 *
 * TEST INFRASTRUCTURE ONLY. This library restates the reference algorithm
 * (hgrecco/fpm-rs 0.2.0-beta.2) in plain C with complex128 arithmetic so that
 * the CUDA product path can be checked against it. Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg load it; the product
 * library never links or calls it.
 *
 * Every array is row-major and C-contiguous. Complex arrays are interleaved
 * (re, im) doubles. Shapes are (height, width).
 */
#ifndef FPM_ORACLE_H
#define FPM_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes mirror the reference error taxonomy (src/error.rs). */
enum {
    ORC_OK = 0,
    ORC_INVALID_SHAPE = 1,
    ORC_INVALID_PARAMETER = 2,
    ORC_INVALID_MODEL = 3,
    ORC_INVALID_MEASUREMENTS = 4,
    ORC_LENGTH_MISMATCH = 5,
    ORC_FRAME_OUT_OF_RANGE = 6,
    ORC_NUMERICAL = 7,
    ORC_UNSUPPORTED = 8
};

enum { ORC_SHAPE_EXACT = 0, ORC_SHAPE_MINIMUM = 1, ORC_SHAPE_SMOOTH = 2, ORC_SHAPE_POW2 = 3 };

enum { ORC_LOSS_AMPLITUDE_MSE = 0, ORC_LOSS_INTENSITY_MSE = 1, ORC_LOSS_POISSON_NLL = 2, ORC_LOSS_HUBER = 3 };

enum { ORC_ALG_AP = 0, ORC_ALG_FPIE = 1, ORC_ALG_MPIE = 2, ORC_ALG_EPRY = 3, ORC_ALG_GD = 4, ORC_ALG_ADAPTIVE_AP = 5 };

enum {
    ORC_SCHEDULE_SEQUENTIAL = 0,
    ORC_SCHEDULE_BRIGHTFIELD_FIRST = 1,
    ORC_SCHEDULE_SPIRAL_OUT = 2,
    ORC_SCHEDULE_SNR_WEIGHTED = 3
};

typedef struct {
    double wavelength_vacuum_m, objective_na, magnification, camera_pixel_size;
    double illumination_refractive_index, objective_medium_refractive_index;
    int32_t has_defocus;
    double defocus_distance;
    int32_t has_aberration;
    double astigmatism, coma, spherical, edge_apodization;
} orc_optics;

/* Compiled image-plane model produced by orc_compile. Arrays are caller-owned
 * and sized by the caller from (h, w) and the source count. */
typedef struct {
    int32_t h, w, mh, mw, sources;
    int64_t *start_row, *start_col;
    double *off_row, *off_col;
    double *pupil;          /* h*w complex */
    uint8_t *support;       /* h*w */
    double dkx, dky, low_res_pixel_size, high_res_pixel_size;
} orc_compiled;

/* One reconstruction problem (non-multiplexed model, frames == sources). */
typedef struct {
    int32_t h, w, mh, mw, frames;
    const int64_t *start_row, *start_col;
    const double *off_row, *off_col;   /* NULL: integer crops */
    const double *pupil;               /* h*w complex */
    const uint8_t *support;            /* h*w */
    const double *gains;               /* NULL or frames */
    const double *background;          /* NULL, h*w or frames*h*w */
    int64_t background_len;
    const double *kx, *ky;             /* per source; used by sorted schedules */
    const double *data;                /* frames*h*w */
    const double *weights;             /* NULL or frames */
    const uint8_t *masks;              /* NULL or frames*h*w */
} orc_problem;

typedef struct {
    int32_t algorithm, iterations, batch_size, loss_type, schedule;
    double object_step, epsilon;
    double stability;                  /* FPIE / mPIE rPIE blend */
    int32_t momentum_interval;
    double momentum_friction, momentum_feedback;
    int32_t recover_pupil, constrain_pupil;
    double pupil_step;
    int32_t recover_gains;
    double gain_step, gain_min, gain_max;
    int32_t recover_background;
    double background_step, background_min, background_max;
    double poisson_truncation_threshold;   /* GD: 0 disables the truncation gate */
    double progress_threshold, reduction_factor, minimum_object_step;  /* adaptive AP controller */
    double object_tv_weight, object_tv_epsilon;   /* GD object TV regulariser (weight 0: off) */
    double pupil_smoothing_weight;                /* GD pupil quadratic smoothing (0: off) */
    int32_t recover_illumination;                 /* GD finite-difference source-offset recovery */
    double illumination_step, illumination_finite_difference, illumination_bounds;
    const double *initial_spectrum;               /* optional mh*mw complex start state (ReconstructionState::from_object) */
} orc_params;

/* truncation_accepts (src/algorithms/gradient_descent.rs:1180-1182). */
int32_t orc_truncation_accepts(double predicted, double measured, double scale);

typedef struct {
    double *object_spectrum;  /* mh*mw complex, centred */
    double *pupil;            /* h*w complex */
    double *objectives;       /* iterations */
    double *object;           /* optional mh*mw complex real-space object */
    int32_t status;
    double *illumination_corrections;  /* optional frames*2 (row, column) recovered offset corrections */
    double *frame_gains;               /* optional frames: the state's (recovered) frame gains */
    double *background;                /* optional frames*h*w: the state's (recovered) background, 0 when none */
    double *object_steps;              /* optional [iterations]: the object step each pass used (adaptive AP trace) */
} orc_output;

const char *orc_last_error(void);

int32_t orc_fft2(double *values, int32_t h, int32_t w, int32_t inverse);
int32_t orc_fftshift(const double *src, double *dst, int32_t h, int32_t w);
int32_t orc_ifftshift(const double *src, double *dst, int32_t h, int32_t w);

int32_t orc_next_smooth(int64_t minimum, int64_t *out);
int32_t orc_compile(const orc_optics *optics, int32_t sources, const double *kx, const double *ky,
                    int32_t h, int32_t w, int32_t policy, int32_t exact_mh, int32_t exact_mw,
                    orc_compiled *out);
int32_t orc_suggest_shape(const orc_optics *optics, int32_t sources, const double *kx,
                          const double *ky, int32_t h, int32_t w, int32_t policy, int32_t *mh,
                          int32_t *mw);
int32_t orc_planar_kvectors(const orc_optics *optics, int32_t rows, int32_t cols, double pitch_x,
                            double pitch_y, double ref_col, double ref_row,
                            const double *translation, const double *rotation, double *kx,
                            double *ky);

int32_t orc_extract_patch(const double *spectrum, int32_t mh, int32_t mw, int64_t start_row,
                          int64_t start_col, int32_t h, int32_t w, double off_row, double off_col,
                          double *patch);
int32_t orc_insert_adjoint(double *spectrum, int32_t mh, int32_t mw, int64_t start_row,
                           int64_t start_col, int32_t h, int32_t w, double off_row, double off_col,
                           const double *update, double scale);

int32_t orc_object_spectrum(const double *object, int32_t mh, int32_t mw, double *spectrum);
int32_t orc_state_object(const double *spectrum, int32_t mh, int32_t mw, double *object);
int32_t orc_forward_stack(const orc_problem *problem, const double *spectrum, double *out,
                          int32_t workers);

int32_t orc_momentum_event(double *object, double *velocity, double *anchor, int64_t len,
                           double friction, double feedback);

int32_t orc_run(const orc_problem *problem, const orc_params *params, orc_output *out);
int32_t orc_run_many(int32_t count, const orc_problem *problems, const orc_params *params,
                     orc_output *outputs, int32_t workers);

double orc_complex_nrmse(const double *reference, const double *candidate, int64_t len);

/* One GradientDescent::step over the batch `frames` from the given centred
 * spectrum (mh*mw) and pupil (h*w); writes the stepped state. */
int32_t orc_gd_batch_step(const orc_problem *problem, const orc_params *params, const double *spectrum,
                          const double *pupil, const int32_t *frames, int32_t count, double *spectrum_out,
                          double *pupil_out, double *illumination_gradient_out, double *corrections_inout);
/* canonicalize_object_pupil (src/algorithms/gauge.rs:20-73) in place. */
int32_t orc_canonicalize(const orc_problem *problem, double *spectrum, double *pupil);
/* Mean point loss of one frame over its unmasked pixels (objective.rs:14-46). */
int32_t orc_frame_loss(const orc_problem *problem, const double *spectrum, const double *pupil, int32_t frame,
                       int32_t loss, double *out);

/* apply_complex_tv_step / apply_quadratic_smoothing_step
 * (src/algorithms/regularization.rs:5-80) on h*w complex values, in place. */
int32_t orc_complex_tv_step(double *values, int32_t h, int32_t w, double weight, double epsilon);
int32_t orc_quadratic_smoothing_step(double *values, int32_t h, int32_t w, double weight);

/* Narrowband spectral problem (src/model/spectral.rs:46-54,
 * src/experiment/spectral.rs:44-70): channel kernels on one common grid and a
 * canonical sparse detector plan. Channel c's local frames are sources
 * [source_offset(c), source_offset(c) + channel_sources[c]) of the
 * concatenated per-source arrays. */
typedef struct {
    int32_t h, w, mh, mw;
    int32_t channels;
    int32_t shared_object;               /* 1: ObjectCoupling::SharedComplex */
    const int32_t *channel_sources;      /* [channels] */
    const int64_t *start_row, *start_col;
    const double *off_row, *off_col;     /* NULL: integer crops */
    const double *frame_gains;           /* NULL (unit) or concatenated per source */
    const double *pupils;                /* channels*h*w complex */
    int32_t exposures;
    const int32_t *contribution_offsets; /* [exposures + 1] */
    const int32_t *contribution_channel, *contribution_local;
    const double *contribution_weight;
    const double *exposure_gain, *exposure_background;  /* [exposures] */
    const double *data;                  /* exposures*h*w */
    const double *weights;               /* NULL or exposures */
    const uint8_t *masks;                /* NULL or exposures*h*w */
} orc_spectral_problem;

typedef struct {
    int32_t iterations, loss_type;
    double object_step, epsilon;
} orc_spectral_params;

/* SpectralRunner::run with SpectralAlternatingProjection
 * (src/reconstruction/spectral.rs:494-642, src/algorithms/spectral.rs:182-271).
 * order: NULL (sequential) or an exposure permutation used every pass.
 * initial_objects: NULL (measured-amplitude initialisation) or
 * object_count*mh*mw natural-order complex objects. initial_spectra, when not
 * NULL, replaces both: centred spectra to continue from, with
 * completed_iterations passes already done. spectra receives object_count
 * centred spectra; objectives one value per executed pass. */
int32_t orc_spectral_run(const orc_spectral_problem *problem, const orc_spectral_params *params,
                         const int32_t *order, const double *initial_objects, const double *initial_spectra,
                         int32_t completed_iterations, double *spectra, double *objectives);

/* SpectralImagePlaneModel::forward_intensity (src/model/spectral.rs:400-446)
 * for every exposure: out is exposures*h*w. */
int32_t orc_spectral_forward(const orc_spectral_problem *problem, const double *spectra, double *out);

#ifdef __cplusplus
}
#endif

#endif
