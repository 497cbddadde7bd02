// Rust binding of include/fpm_gpu.h: the declarations a maintainer adds as
// src/backend/gpu.rs in fpm-rs to reach this library from GpuBackend
// (dispatch at ReconstructionAlgorithm::run / Runner::run,
// src/reconstruction/runner.rs:76-285, when the backend reports
// preferred_memory == Device, src/backend/traits.rs:24-39). Every #[repr(C)]
// struct lists the C struct's fields in the same order with the same types.
#![allow(non_camel_case_types, dead_code)]

use std::os::raw::c_char;

#[repr(C)] pub struct FpmOptics { pub wavelength_vacuum_m: f64, pub objective_na: f64, pub magnification: f64,
    pub camera_pixel_size: f64, pub illumination_refractive_index: f64,
    pub objective_medium_refractive_index: f64, pub has_defocus: i32, pub defocus_distance: f64,
    pub has_aberration: i32, pub astigmatism: f64, pub coma: f64, pub spherical: f64, pub edge_apodization: f64 }
#[repr(C)] pub struct FpmModelDesc { pub image_height: i32, pub image_width: i32, pub recon_height: i32,
    pub recon_width: i32, pub sources: i32, pub crop_start_row: *const i64, pub crop_start_col: *const i64,
    pub offset_row: *const f64, pub offset_col: *const f64, pub pupil: *const f64, pub support: *const u8,
    pub frame_gains: *const f64, pub background: *const f64, pub background_len: i64,
    pub kx: *const f64, pub ky: *const f64 }
#[repr(C)] pub struct FpmMeasurementDesc { pub frames: i32, pub measurements: *const f64,
    pub frame_weights: *const f64, pub masks: *const u8 }
#[repr(C)] pub struct FpmAlgorithmParams { pub algorithm: i32, pub iterations: i32, pub batch_size: i32,
    pub loss_type: i32, pub schedule: i32, pub object_step: f64, pub epsilon: f64, pub stability: f64,
    pub momentum_interval: i32, pub momentum_friction: f64, pub momentum_feedback: f64,
    pub recover_pupil: i32, pub constrain_pupil_support: i32, pub pupil_step: f64,
    pub recover_frame_gains: i32, pub recover_background: i32, pub poisson_truncation: i32,
    pub poisson_truncation_threshold: f64, pub progress_threshold: f64, pub reduction_factor: f64,
    pub minimum_object_step: f64, pub object_tv_weight: f64, pub object_tv_epsilon: f64,
    pub pupil_smoothing_weight: f64, pub recover_illumination: i32, pub illumination_step: f64,
    pub illumination_finite_difference: f64, pub maximum_illumination_correction: f64,
    pub compensated_accumulation: i32, pub gain_step: f64, pub gain_min: f64, pub gain_max: f64,
    pub background_step: f64, pub background_min: f64, pub background_max: f64 }
#[repr(C)] pub struct FpmResultDesc { pub object: *mut f64, pub object_spectrum: *mut f64,
    pub pupil: *mut f64, pub objectives: *mut f64, pub completed_iterations: i32,
    pub illumination_corrections: *mut f64, pub frame_gains: *mut f64, pub background: *mut f64 }
pub enum FpmContext {}
pub enum FpmProblem {}
pub enum FpmPlan {}
pub enum FpmServer {}
#[link(name = "fpm_gpu")]
extern "C" {
    pub fn fpm_create(ctx: *mut *mut FpmContext, device: i32) -> i32;
    pub fn fpm_destroy(ctx: *mut FpmContext) -> i32;
    pub fn fpm_last_error(ctx: *const FpmContext, buf: *mut c_char, len: usize) -> i32;
    pub fn fpm_problem_create(ctx: *mut FpmContext, model: *const FpmModelDesc,
        meas: *const FpmMeasurementDesc, out: *mut *mut FpmProblem) -> i32;
    pub fn fpm_problem_create_batch(ctx: *mut FpmContext, n: i32, models: *const FpmModelDesc,
        meas: *const FpmMeasurementDesc, out: *mut *mut FpmProblem) -> i32;
    pub fn fpm_problem_destroy(p: *mut FpmProblem) -> i32;
    pub fn fpm_run(ctx: *mut FpmContext, p: *mut FpmProblem, a: *const FpmAlgorithmParams,
        r: *mut FpmResultDesc) -> i32;
    pub fn fpm_run_batch(ctx: *mut FpmContext, n: i32, p: *const *mut FpmProblem,
        a: *const FpmAlgorithmParams, r: *mut FpmResultDesc) -> i32;
    pub fn fpm_run_batch_host(ctx: *mut FpmContext, n: i32, models: *const FpmModelDesc,
        meas: *const FpmMeasurementDesc, a: *const FpmAlgorithmParams, r: *mut FpmResultDesc,
        out: *mut *mut FpmProblem) -> i32;
    pub fn fpm_fft2(ctx: *mut FpmContext, values: *mut f64, h: i32, w: i32, inverse: i32) -> i32;
    pub fn fpm_run_batch_resumable(ctx: *mut FpmContext, n: i32, p: *const *mut FpmProblem,
        a: *const FpmAlgorithmParams, resume: *const FpmStateDesc, r: *mut FpmResultDesc,
        capture: *mut FpmStateDesc) -> i32;
    pub fn fpm_simulate_stack(ctx: *mut FpmContext, model: *const FpmModelDesc, object: *const f64,
        camera: *const FpmCameraDesc, seed: u64, counts: *mut f64) -> i32;
    pub fn fpm_spectral_run(ctx: *mut FpmContext, model: *const FpmSpectralModelDesc,
        m: *const FpmMeasurementDesc, p: *const FpmSpectralParams, order: *const i32,
        initial_objects: *const f64, resume_spectra: *const f64, completed: i32,
        objects: *mut f64, object_spectra: *mut f64, objectives: *mut f64) -> i32;
    pub fn fpm_spectral_run_batch(ctx: *mut FpmContext, n: i32, models: *const FpmSpectralModelDesc,
        m: *const FpmMeasurementDesc, p: *const FpmSpectralParams, r: *mut FpmSpectralResultDesc) -> i32;
    pub fn fpm_spectral_forward(ctx: *mut FpmContext, model: *const FpmSpectralModelDesc,
        spectra: *const f64, intensities: *mut f64) -> i32;
    pub fn fpm_run_batch_submit(ctx: *mut FpmContext, n: i32, p: *const *mut FpmProblem,
        a: *const FpmAlgorithmParams, r: *mut FpmResultDesc, job: *mut *mut FpmJob) -> i32;
    pub fn fpm_spectral_run_batch_submit(ctx: *mut FpmContext, n: i32, models: *const FpmSpectralModelDesc,
        m: *const FpmMeasurementDesc, p: *const FpmSpectralParams, r: *mut FpmSpectralResultDesc,
        job: *mut *mut FpmJob) -> i32;
    pub fn fpm_job_poll(job: *mut FpmJob, done: *mut i32) -> i32;
    pub fn fpm_job_wait(job: *mut FpmJob) -> i32;
    pub fn fpm_job_stats(job: *mut FpmJob, stats: *mut FpmRunStats) -> i32;
    pub fn fpm_job_destroy(job: *mut FpmJob) -> i32;
    pub fn fpm_global_last_error() -> *const c_char;
    pub fn fpm_planar_led_kvectors(optics: *const FpmOptics, rows: i32, cols: i32, pitch_x: f64, pitch_y: f64,
        reference_col: f64, reference_row: f64, translation: *const f64, rotation_rad: *const f64,
        kx: *mut f64, ky: *mut f64) -> i32;
    pub fn fpm_suggest_shape(optics: *const FpmOptics, sources: i32, kx: *const f64, ky: *const f64,
        image_height: i32, image_width: i32, policy: i32, recon_height: *mut i32, recon_width: *mut i32) -> i32;
    pub fn fpm_intensity_loss(predicted: *const f64, measured: *const f64, count: i64, loss_type: i32,
        out: *mut f64) -> i32;
    pub fn fpm_compile_model(optics: *const FpmOptics, sources: i32, kx: *const f64, ky: *const f64,
        image_height: i32, image_width: i32, policy: i32, recon_height: *mut i32, recon_width: *mut i32,
        start_row: *mut i64, start_col: *mut i64, offset_row: *mut f64, offset_col: *mut f64, pupil: *mut f64,
        support: *mut u8, dkx: *mut f64, dky: *mut f64) -> i32;
    pub fn fpm_fft2_noalloc(ctx: *mut FpmContext, values: *mut f64, h: i32, w: i32, inverse: i32) -> i32;
    pub fn fpm_forward_stack(ctx: *mut FpmContext, model: *const FpmModelDesc, object: *const f64,
        intensities: *mut f64) -> i32;
    pub fn fpm_last_run_stats(ctx: *const FpmContext, stats: *mut FpmRunStats) -> i32;
    pub fn fpm_plan_create(ctx: *mut FpmContext, n: i32, p: *const *mut FpmProblem, a: *const FpmAlgorithmParams,
        plan: *mut *mut FpmPlan) -> i32;
    pub fn fpm_plan_launch(plan: *mut FpmPlan) -> i32;
    pub fn fpm_plan_wait(plan: *mut FpmPlan) -> i32;
    pub fn fpm_plan_collect(plan: *mut FpmPlan, r: *mut FpmResultDesc) -> i32;
    pub fn fpm_plan_destroy(plan: *mut FpmPlan) -> i32;
    pub fn fpm_set_engine_grid(ctx: *mut FpmContext, n: i32, clusters: i32) -> i32;
    pub fn fpm_engine_max_clusters(ctx: *mut FpmContext, n: i32, clusters: *mut i32) -> i32;
    pub fn fpm_set_engine_shape(ctx: *mut FpmContext, n: i32, shape: i32) -> i32;
    pub fn fpm_set_engine_ctas(ctx: *mut FpmContext, n: i32, ctas: i32) -> i32;
    pub fn fpm_server_create(ctx: *mut FpmContext, config: *const FpmServerConfig, server: *mut *mut FpmServer) -> i32;
    pub fn fpm_server_submit(server: *mut FpmServer, model: *const FpmModelDesc, m: *const FpmMeasurementDesc,
        a: *const FpmAlgorithmParams, r: *mut FpmResultDesc, request: *mut u64) -> i32;
    pub fn fpm_server_poll(server: *mut FpmServer, request: u64, done: *mut i32) -> i32;
    pub fn fpm_server_wait(server: *mut FpmServer, request: u64, info: *mut FpmRequestInfo) -> i32;
    pub fn fpm_server_stats_get(server: *mut FpmServer, stats: *mut FpmServerStats) -> i32;
    pub fn fpm_server_destroy(server: *mut FpmServer) -> i32;
}
#[repr(C)] pub struct FpmJob { _opaque: [u8; 0] }
#[repr(C)] pub struct FpmRunStats { pub kernel_launches: i32, pub engine_launches: i32, pub run_ms: f64,
    pub engine_ms_sum: f64, pub engine_span_ms: f64, pub engine_bytes: f64, pub buckets: i32,
    pub bucket_size: [i32; 8], pub bucket_tiles: [i32; 8], pub bucket_end_ms: [f64; 8],
    pub host_first_launch_ms: f64, pub host_scan_ms: f64, pub host_upload_ms: f64, pub host_call_ms: f64,
    pub host_chunks: i32, pub host_done_tiles: [i32; 16], pub host_done_ms: [f64; 16] }
#[repr(C)] pub struct FpmSpectralModelDesc { pub channels: i32, pub channel_models: *const FpmModelDesc,
    pub object_coupling: i32, pub exposures: i32, pub contribution_offsets: *const i32,
    pub contribution_channel: *const i32, pub contribution_local_frame: *const i32,
    pub contribution_weight: *const f64, pub exposure_gain: *const f64, pub exposure_background: *const f64 }
#[repr(C)] pub struct FpmSpectralParams { pub iterations: i32, pub batch_size: i32, pub loss_type: i32,
    pub object_step: f64, pub epsilon: f64 }
#[repr(C)] pub struct FpmSpectralResultDesc { pub objects: *mut f64, pub object_spectra: *mut f64,
    pub objectives: *mut f64 }
#[repr(C)] pub struct FpmStateDesc { pub completed_iterations: i32, pub momentum_counter: i32,
    pub object_spectrum: *mut f64, pub pupil: *mut f64, pub velocity: *mut f64, pub anchor: *mut f64,
    pub objectives: *mut f64, pub illumination_corrections: *mut f64 }
#[repr(C)] pub struct FpmCameraDesc { pub photons_per_pixel: f64, pub gain_counts_per_electron: f64,
    pub offset_counts: f64, pub read_noise_electrons: f64, pub dark_current_electrons: f64,
    pub shot_noise: i32, pub quantize: i32, pub maximum_count: f64, pub pixel_sensitivity: *const f64,
    pub bad_pixels: *const i64, pub bad_pixel_count: i64, pub bad_pixel_value: f64 }
#[repr(C)] pub struct FpmServerConfig { pub hbm_budget_bytes: i64, pub max_batch: i32, pub batch_window_ms: f64,
    pub max_queue: i64 }
#[repr(C)] pub struct FpmRequestInfo { pub submit_ms: f64, pub admit_ms: f64, pub start_ms: f64, pub done_ms: f64,
    pub footprint_bytes: i64, pub status: i32, pub message: [c_char; 256] }
#[repr(C)] pub struct FpmServerStats { pub submitted: i64, pub admitted: i64, pub completed: i64, pub rejected: i64,
    pub batches: i64, pub in_use_bytes: i64, pub peak_bytes: i64, pub waiting: i64, pub in_flight_batches: i64 }
