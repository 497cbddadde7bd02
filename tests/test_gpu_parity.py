"""GPU parity: the CUDA path through the C ABI against the FP64 oracle.

Tolerances: complex NRMSE (global-phase aligned, the reference's
complex_nrmse) <= 1e-4 for reconstructed objects and EPRY pupils after the
stated iteration count; FP64 device kernels (fft2) to 1e-12; the FP32 forward
stack to 1e-5 relative; per-iteration objectives to 1e-4 relative. Integer
work (crop origins, frame order) is bit-exact and checked on the host.
"""

from __future__ import annotations

import numpy as np
import pytest

import helpers
import oracle
import workloads as W

pytestmark = pytest.mark.gpu

NRMSE = 1e-4


@pytest.fixture(scope="module")
def fpm(native_library):
    import fpm_rs

    return fpm_rs


def _objective_close(gpu, cpu, rtol=1e-4):
    gpu = np.asarray(gpu)
    cpu = np.asarray(cpu)
    assert gpu.shape == cpu.shape
    assert np.all(np.abs(gpu - cpu) <= rtol * np.abs(cpu) + 1e-12), (gpu, cpu)


@pytest.mark.parametrize("shape", [(7, 9), (16, 16), (42, 42), (96, 96), (375, 375), (729, 729), (256, 256)])
def test_fft2_matches_reference_convention(fpm, shape):
    rng = np.random.default_rng(3)
    values = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    forward = fpm.fft2(values)
    expected = oracle.fft2(values)
    assert np.abs(forward - expected).max() <= 1e-12 * max(1.0, np.abs(expected).max())
    back = fpm.fft2(forward, inverse=True)
    assert np.abs(back - values).max() <= 1e-10


def test_fft2_constant_object_known_answer(fpm):
    # tests/forward_model_tests.rs:75-101: forward normalisation by 1/N.
    spectrum = fpm.fft2(np.full((16, 16), 2.0 + 0j))
    assert abs(spectrum[0, 0] - 2.0) < 1e-12
    assert np.abs(spectrum.ravel()[1:]).max() < 1e-12


@pytest.mark.parametrize("n,side", [(32, 3), (64, 5), (128, 5), (256, 3)])
def test_forward_stack_matches_oracle(fpm, n, side):
    model, omodel = helpers.planar_model(fpm, side, n)
    obj = W.smooth_random_object(model.reconstruction_shape, 17)
    gpu = fpm.forward_intensities(model, obj)
    cpu = oracle.forward_stack(oracle.Problem(omodel, None), oracle.object_spectrum(obj), workers=8)
    assert np.abs(gpu - cpu).max() <= 1e-5 * np.abs(cpu).max()


def _run_both(fpm, algorithm_gpu, name, kw, model, omodel, data, gains=None, weights=None, masks=None,
              background=None, schedule="sequential"):
    problem = fpm.ReconstructionProblem(data, model, frame_weights=weights, masks=masks)
    result = algorithm_gpu.run(problem, schedule=schedule)
    expected = oracle.run(oracle.Problem(omodel, data, weights=weights, masks=masks, gains=gains,
                                         background=background), name, schedule=schedule, **kw)
    return result, expected


def test_ap_quickstart_config(fpm):
    """Plain AP, README quickstart geometry: 3x3 LEDs, 32x32 frames, M=42, 20 iterations, ideal camera."""
    model, omodel, data, truth, _ = helpers.simulated(fpm, 3, 32, seed=1234)
    assert model.reconstruction_shape == (42, 42)
    result, expected = _run_both(fpm, fpm.AlternatingProjection(iterations=20), "ap", dict(iterations=20),
                                 model, omodel, data)
    assert oracle.complex_nrmse(expected["object"], result.object) <= NRMSE
    assert oracle.complex_nrmse(expected["object_spectrum"], result.object_spectrum) <= NRMSE
    _objective_close([t[1] for t in result.trace], expected["objectives"])
    assert result.trace[-1][1] < result.trace[0][1]


@pytest.mark.parametrize("alg,kw", [
    ("ap", dict(iterations=6)),
    ("fpie", dict(iterations=6)),
    ("mpie", dict(iterations=6, momentum_interval=7)),
    ("epry", dict(iterations=6)),
    ("gd", dict(iterations=6)),
])
@pytest.mark.parametrize("n,side", [(32, 5), (64, 5)])
def test_algorithms_small(fpm, alg, kw, n, side):
    model, omodel, data, truth, gains = helpers.simulated(fpm, side, n, seed=7, photons=1e4)
    cls = {"ap": fpm.AlternatingProjection, "fpie": fpm.Fpie, "mpie": fpm.Mpie, "epry": fpm.Epry,
           "gd": fpm.GradientDescent}[alg]
    result, expected = _run_both(fpm, cls(**kw), alg, kw, model, omodel, data, gains=gains)
    assert oracle.complex_nrmse(expected["object"], result.object) <= NRMSE
    _objective_close([t[1] for t in result.trace], expected["objectives"])
    if alg == "epry":
        assert oracle.complex_nrmse(expected["pupil"], result.recovered_pupil) <= NRMSE


@pytest.mark.parametrize("alg,kw", [
    ("ap", dict(iterations=3)),
    ("fpie", dict(iterations=3)),
    ("mpie", dict(iterations=3, momentum_interval=7)),
    ("epry", dict(iterations=3)),
])
def test_algorithms_256(fpm, alg, kw):
    """256-point tiles: 16-row CTAs in 16-CTA clusters."""
    model, omodel, data, truth, gains = helpers.simulated(fpm, 5, 256, seed=8, photons=1e4)
    cls = {"ap": fpm.AlternatingProjection, "fpie": fpm.Fpie, "mpie": fpm.Mpie, "epry": fpm.Epry}[alg]
    result, expected = _run_both(fpm, cls(**kw), alg, kw, model, omodel, data, gains=gains)
    assert oracle.complex_nrmse(expected["object"], result.object) <= NRMSE
    _objective_close([t[1] for t in result.trace], expected["objectives"])
    if alg == "epry":
        assert oracle.complex_nrmse(expected["pupil"], result.recovered_pupil) <= NRMSE


def test_mpie_full_tile_bench_config(fpm):
    """The bench's largest tile: 256 x 256 frames, 15x15 LEDs (M=729), mPIE
    defaults (momentum every 30 frames), Poisson 1e4."""
    model, omodel, data, truth, gains = helpers.simulated(fpm, 15, 256, seed=9, photons=1e4)
    assert model.reconstruction_shape == (729, 729)
    result, expected = _run_both(fpm, fpm.Mpie(iterations=2), "mpie", dict(iterations=2), model, omodel, data,
                                 gains=gains)
    assert oracle.complex_nrmse(expected["object"], result.object) <= NRMSE
    _objective_close([t[1] for t in result.trace], expected["objectives"])


def test_masks_background_256(fpm):
    """Raw measurement form (background present) and amplitude form with
    masks at 256 x 256."""
    model, omodel, data, truth, gains = helpers.simulated(fpm, 3, 256, seed=22, photons=3e3)
    rng = np.random.default_rng(6)
    masks = (rng.random(data.shape) > 0.15).astype(np.uint8)
    weights = np.ones(data.shape[0])
    weights[2] = 0.0
    result, expected = _run_both(fpm, fpm.Mpie(iterations=2), "mpie", dict(iterations=2), model, omodel, data,
                                 gains=gains, weights=weights, masks=masks)
    assert oracle.complex_nrmse(expected["object"], result.object) <= NRMSE
    background = np.full(256 * 256, 2.0)
    model_bg = model._replace(background=background)
    result, expected = _run_both(fpm, fpm.AlternatingProjection(iterations=2), "ap", dict(iterations=2), model_bg,
                                 omodel, data + 2.0, gains=gains, weights=weights, masks=masks, background=background)
    assert oracle.complex_nrmse(expected["object"], result.object) <= NRMSE
    _objective_close([t[1] for t in result.trace], expected["objectives"])


def test_mpie_epry_pupil_config(fpm):
    """mPIE and EPRY, 13x13 LEDs, 128x128 frames (M=336), Zernike true pupil, Poisson 5e3."""
    model, omodel, data, truth, gains = helpers.simulated(fpm, 13, 128, seed=1, photons=5e3, pupil_seed=11)
    assert model.reconstruction_shape == (336, 336)
    for name, algo, kw in (("mpie", fpm.Mpie(iterations=3), dict(iterations=3)),
                           ("epry", fpm.Epry(iterations=3), dict(iterations=3))):
        result, expected = _run_both(fpm, algo, name, kw, model, omodel, data, gains=gains)
        assert oracle.complex_nrmse(expected["object"], result.object) <= NRMSE, name
        _objective_close([t[1] for t in result.trace], expected["objectives"])
        if name == "epry":
            assert oracle.complex_nrmse(expected["pupil"], result.recovered_pupil) <= NRMSE


def test_mpie_epry_pupil_recovery_128_full_50_iterations(fpm):
    """The pupil-recovery workload at its full 50 iterations: mPIE and EPRY
    with pupil recovery, 13x13 LEDs, 128x128 frames (M=336), Zernike true
    pupil (seed 11), Poisson 5e3. Object (and EPRY pupil) NRMSE <= 1e-4 vs FP64."""
    from concurrent.futures import ThreadPoolExecutor

    model, omodel, data, truth, gains = helpers.simulated(fpm, 13, 128, seed=1, photons=5e3, pupil_seed=11)
    oproblem = oracle.Problem(omodel, data, gains=gains)
    with ThreadPoolExecutor(max_workers=2) as pool:
        futures = {name: pool.submit(oracle.run, oproblem, name, iterations=50) for name in ("mpie", "epry")}
        problem = fpm.ReconstructionProblem(data, model)
        got = {"mpie": fpm.Mpie(iterations=50).run(problem), "epry": fpm.Epry(iterations=50).run(problem)}
        compensated = {"mpie": fpm.Mpie(iterations=50).compensated().run(problem),
                       "epry": fpm.Epry(iterations=50).compensated().run(problem)}
        expected = {name: f.result() for name, f in futures.items()}
    for runs in (got, compensated):
        for name in ("mpie", "epry"):
            assert oracle.complex_nrmse(expected[name]["object"], runs[name].object) <= NRMSE, name
            _objective_close([t[1] for t in runs[name].trace], expected[name]["objectives"])
        assert oracle.complex_nrmse(expected["epry"]["pupil"], runs["epry"].recovered_pupil) <= NRMSE


def test_gradient_descent_256_full_100_iterations(fpm):
    """The 256-point GD workload at its full 100 iterations: 256x256 frames,
    15x15 LEDs (M=729), Poisson 1e4 at the bright-field peak, seed 7."""
    model, omodel, data, truth, gains = helpers.simulated(fpm, 15, 256, seed=7, photons=1e4)
    result, expected = _run_both(fpm, fpm.GradientDescent(iterations=100), "gd", dict(iterations=100), model, omodel,
                                 data, gains=gains)
    assert oracle.complex_nrmse(expected["object"], result.object) <= NRMSE
    _objective_close([t[1] for t in result.trace], expected["objectives"])
    # The same run with compensated accumulation of the frame updates.
    compensated = fpm.GradientDescent(iterations=100).compensated().run(fpm.ReconstructionProblem(data, model))
    assert oracle.complex_nrmse(expected["object"], compensated.object) <= NRMSE
    _objective_close([t[1] for t in compensated.trace], expected["objectives"])


def test_gradient_descent_full_tile(fpm):
    """Wirtinger GD on one 256x256 tile with 15x15 LEDs (M=729), Poisson 1e4, 2 iterations."""
    model, omodel, data, truth, gains = helpers.simulated(fpm, 15, 256, seed=7, photons=1e4)
    assert model.reconstruction_shape == (729, 729)
    result, expected = _run_both(fpm, fpm.GradientDescent(iterations=2), "gd", dict(iterations=2), model, omodel,
                                 data, gains=gains)
    assert oracle.complex_nrmse(expected["object"], result.object) <= NRMSE
    _objective_close([t[1] for t in result.trace], expected["objectives"])


@pytest.mark.parametrize("n,side,batch", [(32, 5, 4), (64, 3, 9), (128, 3, 2)])
def test_gradient_descent_mini_batches(fpm, n, side, batch):
    """GD with batch_size > 1: gradients of a batch accumulate, the object
    moves once per batch by object_step / active frames
    (src/algorithms/gradient_descent.rs:405-640); zero-weight frames count
    toward batch boundaries but not toward the active frames."""
    model, omodel, data, truth, gains = helpers.simulated(fpm, side, n, seed=41, photons=1e4)
    weights = np.ones(data.shape[0])
    weights[1] = 0.0
    weights[3] = 0.5
    for loss in ("amplitude_mse", "poisson_nll"):
        algo = fpm.GradientDescent(iterations=3, batch_size=batch, loss_type=loss)
        result, expected = _run_both(fpm, algo, "gd", dict(iterations=3, batch_size=batch, loss_type=loss), model,
                                     omodel, data, gains=gains, weights=weights)
        assert oracle.complex_nrmse(expected["object"], result.object) <= NRMSE, loss
        _objective_close([t[1] for t in result.trace], expected["objectives"])
        # Compensated accumulation of the batch gradient gives the same answer.
        problem = fpm.ReconstructionProblem(data, model, frame_weights=weights)
        compensated = fpm.GradientDescent(iterations=3, batch_size=batch, loss_type=loss).compensated().run(problem)
        assert oracle.complex_nrmse(expected["object"], compensated.object) <= NRMSE, loss


@pytest.mark.parametrize("n,side,batch,threshold", [(32, 5, 5, 25.0), (64, 3, 1, 2.0), (128, 3, 9, 4.0)])
def test_gradient_descent_poisson_truncation(fpm, n, side, batch, threshold):
    """Poisson truncation (src/algorithms/gradient_descent.rs:701-792,1180-1182):
    per batch, a forward-only pass gives the gate scale; pixels with
    |y - p| > scale * sqrt(p) leave the gradient but stay in the objective."""
    model, omodel, data, truth, gains = helpers.simulated(fpm, side, n, seed=43, photons=3e3)
    kw = dict(iterations=3, batch_size=batch, loss_type="poisson_nll", poisson_truncation_threshold=threshold)
    result, expected = _run_both(fpm, fpm.GradientDescent(**kw), "gd", kw, model, omodel, data, gains=gains)
    assert oracle.complex_nrmse(expected["object"], result.object) <= NRMSE
    _objective_close([t[1] for t in result.trace], expected["objectives"])
    plain = oracle.run(oracle.Problem(omodel, data, gains=gains), "gd", iterations=3, batch_size=batch,
                       loss_type="poisson_nll")
    if threshold < 10.0:
        # The gate rejects pixels at this threshold: results differ from plain GD.
        assert oracle.complex_nrmse(plain["object"], expected["object"]) > 10 * NRMSE


def test_poisson_truncation_validation(fpm):
    model, omodel = helpers.planar_model(fpm, 3, 32)
    problem = fpm.ReconstructionProblem(np.ones((model.frame_count, 32, 32)), model)
    with pytest.raises(fpm.InvalidParameterError):
        fpm.GradientDescent(iterations=1, poisson_truncation_threshold=25.0).run(problem)
    with pytest.raises(fpm.InvalidParameterError):
        fpm.GradientDescent(iterations=1, loss_type="poisson_nll", poisson_truncation_threshold=-1.0).run(problem)


def test_masks_weights_background(fpm):
    """Masked pixels, a zero-weight frame and a broadcast background (AP and GD)."""
    model, omodel, data, truth, gains = helpers.simulated(fpm, 5, 32, seed=21, photons=2e3)
    rng = np.random.default_rng(5)
    masks = (rng.random(data.shape) > 0.1).astype(np.uint8)
    weights = np.ones(data.shape[0])
    weights[3] = 0.0
    weights[7] = 0.5
    background = np.full(32 * 32, 3.0)
    data = data + 3.0
    model = model._replace(background=background)
    for name, algo in (("ap", fpm.AlternatingProjection(iterations=4)), ("gd", fpm.GradientDescent(iterations=4))):
        result, expected = _run_both(fpm, algo, name, dict(iterations=4), model, omodel, data, gains=gains,
                                     weights=weights, masks=masks, background=background)
        assert oracle.complex_nrmse(expected["object"], result.object) <= NRMSE, name
        _objective_close([t[1] for t in result.trace], expected["objectives"])


@pytest.mark.parametrize("n,side", [(32, 5), (128, 3)])
def test_masks_and_weights_without_background(fpm, n, side):
    """Masks with no background: the device keeps amplitudes, -1 on masked pixels.

    Negative counts (possible after dark subtraction) must clamp to zero
    amplitude exactly as max(I / g, 0) does in the reference."""
    model, omodel, data, truth, gains = helpers.simulated(fpm, side, n, seed=31, photons=3e3)
    rng = np.random.default_rng(8)
    masks = (rng.random(data.shape) > 0.2).astype(np.uint8)
    data = data.copy()
    data[1, :4, :4] = -2.0
    weights = np.ones(data.shape[0])
    weights[2] = 0.0
    weights[4] = 0.25
    for name, algo, kw in (("ap", fpm.AlternatingProjection(iterations=3), dict(iterations=3)),
                           ("mpie", fpm.Mpie(iterations=3, momentum_interval=4), dict(iterations=3, momentum_interval=4)),
                           ("gd", fpm.GradientDescent(iterations=3), dict(iterations=3))):
        result, expected = _run_both(fpm, algo, name, kw, model, omodel, data, gains=gains, weights=weights,
                                     masks=masks)
        assert oracle.complex_nrmse(expected["object"], result.object) <= NRMSE, name
        _objective_close([t[1] for t in result.trace], expected["objectives"])


def test_batched_upload_matches_single_uploads(fpm):
    """fpm_problem_create_batch gives the same problems as one-by-one creation."""
    cases = [helpers.simulated(fpm, side, n, seed=seed, photons=1e4)
             for n, side, seed in ((32, 3, 11), (64, 3, 12), (32, 5, 13))]
    algo = fpm.Fpie(iterations=2)
    single = []
    for model, _, data, _, _ in cases:
        p = fpm.ReconstructionProblem(data, model)
        p.device_handle()
        single.append(algo.run(p).object)
    batched = [fpm.ReconstructionProblem(data, model) for model, _, data, _, _ in cases]
    from fpm_rs import reconstruction

    reconstruction.upload(batched)  # fpm_problem_create_batch
    results = fpm.run_batch(algo, batched)
    for a, r in zip(single, results):
        assert np.array_equal(a, r.object)


def test_host_input_batch_matches_resident_batch(fpm):
    """fpm_run_batch_host (copies overlapped with the runs) gives the resident
    path's results bit for bit, and leaves the problems resident."""
    cases = [helpers.simulated(fpm, side, n, seed=seed, photons=1e4)
             for n, side, seed in ((64, 3, 21), (32, 3, 22), (128, 3, 23), (32, 5, 24), (64, 5, 25))]
    algo = fpm.Mpie(iterations=2, momentum_interval=3)
    resident = [fpm.ReconstructionProblem(data, model) for model, _, data, _, _ in cases]
    for p in resident:
        p.device_handle()
    expected = fpm.run_batch(algo, resident)
    host = [fpm.ReconstructionProblem(data, model) for model, _, data, _, _ in cases]
    got = fpm.run_batch(algo, host)  # no handles yet: the host-input path
    for e, g in zip(expected, got):
        assert np.array_equal(e.object, g.object)
        assert np.array_equal(e.object_spectrum, g.object_spectrum)
        assert [t[1] for t in e.trace] == [t[1] for t in g.trace]
    assert all(p._handle is not None for p in host)
    again = fpm.run_batch(algo, host)  # resident now
    for e, g in zip(expected, again):
        assert np.array_equal(e.object, g.object)


def test_host_input_batch_error_returns_no_problems(fpm):
    import ctypes as C
    from fpm_rs import _native as N

    model, _, data, _, _ = helpers.simulated(fpm, 3, 32, seed=26, photons=1e4)
    problems = [fpm.ReconstructionProblem(data, model) for _ in range(2)]
    descs = [p._descriptors() for p in problems]
    bad = data.copy()
    bad[0, 0, 0] = np.nan
    descs[1][1].measurements = N.ptr(bad, C.c_double)
    models = (N.ModelDesc * 2)(*[d[0] for d in descs])
    meas = (N.MeasurementDesc * 2)(*[d[1] for d in descs])
    made = (C.c_void_p * 2)(1, 2)
    ctx = N.context()
    params = fpm.AlternatingProjection(iterations=1)._params("sequential")
    status = N.library().fpm_run_batch_host(ctx.handle, 2, models, meas, C.byref(params), None, made)
    assert status == 4
    buf = C.create_string_buffer(512)
    N.library().fpm_last_error(ctx.handle, buf, len(buf))
    assert buf.value.decode().startswith("problem 1:")
    assert all(h is None for h in made)


def test_batched_upload_error_names_the_problem(fpm):
    import ctypes as C
    from fpm_rs import _native as N

    model, _, data, _, _ = helpers.simulated(fpm, 3, 32, seed=14, photons=1e4)
    problems = [fpm.ReconstructionProblem(data, model) for _ in range(3)]
    descs = [p._descriptors() for p in problems]
    bad = np.full(model.frame_count, -1.0)
    descs[1][1].frame_weights = N.ptr(bad, C.c_double)
    models = (N.ModelDesc * 3)(*[d[0] for d in descs])
    meas = (N.MeasurementDesc * 3)(*[d[1] for d in descs])
    handles = (C.c_void_p * 3)(1, 2, 3)
    ctx = N.context()
    status = N.library().fpm_problem_create_batch(ctx.handle, 3, models, meas, handles)
    assert status == 4  # InvalidMeasurements
    buf = C.create_string_buffer(512)
    N.library().fpm_last_error(ctx.handle, buf, len(buf))
    assert buf.value.decode().startswith("problem 1:")
    assert all(h is None for h in handles)


@pytest.mark.parametrize("schedule", ["brightfield_first", "spiral_out", "snr_weighted"])
def test_schedules(fpm, schedule):
    model, omodel, data, truth, gains = helpers.simulated(fpm, 5, 32, seed=9, photons=1e4)
    result, expected = _run_both(fpm, fpm.Fpie(iterations=3), "fpie", dict(iterations=3), model, omodel, data,
                                 gains=gains, schedule=schedule)
    assert oracle.complex_nrmse(expected["object"], result.object) <= NRMSE


def test_integer_offsets(fpm):
    """k-vectors on exact grid multiples: integer crops, and EPRY's affine ramp gauge is active."""
    optics = fpm.Optics(**W.OPTICS)
    n = 32
    dk = 2 * np.pi / (n * optics.object_pixel_size)
    shifts = [(0, 0), (3, 0), (-3, 0), (0, 3), (0, -3), (2, 2), (-2, 2)]
    k = np.array([[c * dk, r * dk] for r, c in shifts])
    model = fpm.compile_model(optics, fpm.Illumination(fpm.KVectorList(k)), (n, n), (48, 48))
    assert np.all(model.subpixel_offsets == 0.0)
    omodel = oracle.compile_model(W.OPTICS, k[:, 0], k[:, 1], (n, n), (48, 48))
    truth = W.smooth_random_object((48, 48), 4)
    data = oracle.forward_stack(oracle.Problem(omodel, None), oracle.object_spectrum(truth))
    for name, algo in (("ap", fpm.AlternatingProjection(iterations=5)), ("epry", fpm.Epry(iterations=5))):
        result, expected = _run_both(fpm, algo, name, dict(iterations=5), model, omodel, data)
        assert oracle.complex_nrmse(expected["object"], result.object) <= NRMSE, name


def test_deterministic_repeat(fpm):
    """The scatter-add uses no atomics: two runs are bitwise identical."""
    model, omodel, data, truth, gains = helpers.simulated(fpm, 5, 64, seed=2, photons=1e4)
    problem = fpm.ReconstructionProblem(data, model)
    a = fpm.Mpie(iterations=3, momentum_interval=5).run(problem)
    b = fpm.Mpie(iterations=3, momentum_interval=5).run(problem)
    assert np.array_equal(a.object, b.object)
    assert [t[1] for t in a.trace] == [t[1] for t in b.trace]


def test_batch_equals_alone(fpm):
    """Tiles of several sizes in one batch give the same results as alone."""
    problems = []
    for n, side, seed in ((32, 3, 1), (64, 5, 2), (32, 5, 3), (128, 3, 4), (64, 3, 5)):
        model, omodel, data, truth, gains = helpers.simulated(fpm, side, n, seed=seed, photons=1e4)
        problems.append(fpm.ReconstructionProblem(data, model))
    algo = fpm.Mpie(iterations=2, momentum_interval=4)
    batch = fpm.run_batch(algo, problems)
    for p, r in zip(problems, batch):
        alone = algo.run(p)
        assert np.array_equal(alone.object, r.object)


def test_unsupported_and_invalid(fpm):
    model, omodel = helpers.planar_model(fpm, 3, 48)
    data = np.ones((model.frame_count, 48, 48))
    with pytest.raises(fpm.UnsupportedError):
        fpm.AlternatingProjection(iterations=1).run(fpm.ReconstructionProblem(data, model))
    model, omodel = helpers.planar_model(fpm, 3, 32)
    data = np.ones((model.frame_count, 32, 32))
    with pytest.raises(fpm.InvalidParameterError):
        fpm.AlternatingProjection(iterations=1, object_step=-1.0).run(fpm.ReconstructionProblem(data, model))
    with pytest.raises(fpm.InvalidParameterError):
        fpm.Mpie(iterations=1, momentum_friction=1.0).run(fpm.ReconstructionProblem(data, model))


@pytest.mark.parametrize("name,make", [
    ("mpie", lambda fpm: fpm.Mpie(iterations=5, momentum_interval=7)),
    ("epry", lambda fpm: fpm.Epry(iterations=5)),
    ("gd", lambda fpm: fpm.GradientDescent(iterations=5, batch_size=4, loss_type="poisson_nll",
                                           poisson_truncation_threshold=4.0)),
    ("ap", lambda fpm: fpm.AlternatingProjection(iterations=5)),
])
def test_checkpoint_resume_is_bitwise_uninterrupted(fpm, tmp_path, name, make):
    """CheckpointEvery + resume_from (src/reconstruction/checkpoint.rs:38-146):
    the captured complex64 state restores exactly, so runs split at
    checkpoints equal the uninterrupted run bit for bit."""
    model, omodel, data, truth, gains = helpers.simulated(fpm, 5, 64, seed=51, photons=1e4)
    problem = fpm.ReconstructionProblem(data, model)
    straight = make(fpm).run(problem)
    with_callbacks = make(fpm).run(problem, callbacks=[fpm.CheckpointEvery(2, tmp_path)])
    cp = fpm.ReconstructionCheckpoint.load(tmp_path / "checkpoint_00002.json")
    assert cp.completed_iterations == 2 and len(cp.objectives) == 2
    resumed = make(fpm).run(fpm.ReconstructionProblem(data, model), resume_from=cp)
    for other in (with_callbacks, resumed):
        if name == "epry":
            # A restored object/pupil pair is canonicalised again before the
            # run continues (as in the reference); the gauge is idempotent up
            # to rounding.
            assert oracle.complex_nrmse(straight.object, other.object) <= 1e-5
            assert oracle.complex_nrmse(straight.recovered_pupil, other.recovered_pupil) <= 1e-5
            _objective_close([t[1] for t in other.trace], [t[1] for t in straight.trace], rtol=1e-5)
        else:
            assert np.array_equal(straight.object, other.object)
            assert np.array_equal(straight.recovered_pupil, other.recovered_pupil)
            assert [t[1] for t in straight.trace] == [t[1] for t in other.trace]
    cp4 = fpm.ReconstructionCheckpoint.load(tmp_path / "checkpoint_00004.json")
    assert cp4.completed_iterations == 4


def test_checkpoint_resume_rejects_mismatches(fpm, tmp_path):
    model, omodel, data, truth, gains = helpers.simulated(fpm, 3, 32, seed=52, photons=1e4)
    problem = fpm.ReconstructionProblem(data, model)
    fpm.AlternatingProjection(iterations=2).run(problem, callbacks=[fpm.CheckpointEvery(1, tmp_path)])
    cp = fpm.ReconstructionCheckpoint.load(tmp_path / "checkpoint_00001.json")
    with pytest.raises(fpm.InvalidParameterError):
        fpm.Mpie(iterations=3).run(problem, resume_from=cp)
    with pytest.raises(fpm.InvalidParameterError):
        fpm.AlternatingProjection(iterations=0).run(problem, resume_from=cp)


@pytest.mark.parametrize("n,side,threshold", [(32, 5, 0.01), (64, 5, 0.9), (128, 3, 0.5)])
def test_adaptive_alternating_projection(fpm, n, side, threshold):
    """AdaptiveAlternatingProjection: the device controller reads each pass's
    objective from the cluster's partials and shrinks the step like the
    FP64 restatement does."""
    model, omodel, data, truth, gains = helpers.simulated(fpm, side, n, seed=61, photons=1e4)
    kw = dict(iterations=6, progress_threshold=threshold, reduction_factor=0.5, minimum_object_step=0.05)
    algo = fpm.AdaptiveAlternatingProjection(iterations=6, initial_object_step=1.0, progress_threshold=threshold,
                                             reduction_factor=0.5, minimum_object_step=0.05)
    result, expected = _run_both(fpm, algo, "adaptive_ap", kw, model, omodel, data, gains=gains)
    assert oracle.complex_nrmse(expected["object"], result.object) <= NRMSE
    _objective_close([t[1] for t in result.trace], expected["objectives"])
    if threshold >= 0.5:
        plain = oracle.run(oracle.Problem(omodel, data, gains=gains), "ap", iterations=6)
        assert oracle.complex_nrmse(plain["object"], expected["object"]) > 10 * NRMSE  # the step did shrink


def test_adaptive_ap_validation(fpm):
    model, omodel = helpers.planar_model(fpm, 3, 32)
    problem = fpm.ReconstructionProblem(np.ones((model.frame_count, 32, 32)), model)
    with pytest.raises(fpm.InvalidParameterError):
        fpm.AdaptiveAlternatingProjection(iterations=2, reduction_factor=1.0).run(problem)
    with pytest.raises(fpm.InvalidParameterError):
        fpm.AdaptiveAlternatingProjection(iterations=2, minimum_object_step=2.0).run(problem)


@pytest.mark.parametrize("n,side,batch", [(32, 5, 1), (64, 3, 4), (128, 3, 9)])
def test_gradient_descent_pupil_recovery(fpm, n, side, batch):
    """GD with recover_pupil (src/algorithms/gradient_descent.rs:563-656):
    pupil gradient per frame, pupil step per batch, support projection, and
    the object/pupil gauge after every iteration."""
    model, omodel, data, truth, gains = helpers.simulated(fpm, side, n, seed=71, photons=1e4, pupil_seed=5)
    kw = dict(iterations=4, batch_size=batch, recover_pupil=True, pupil_step=0.05)
    result, expected = _run_both(fpm, fpm.GradientDescent(**kw), "gd", kw, model, omodel, data, gains=gains)
    assert oracle.complex_nrmse(expected["object"], result.object) <= NRMSE
    assert oracle.complex_nrmse(expected["pupil"], result.recovered_pupil) <= NRMSE
    _objective_close([t[1] for t in result.trace], expected["objectives"])
    plain = oracle.run(oracle.Problem(omodel, data, gains=gains), "gd", iterations=4, batch_size=batch)
    assert oracle.complex_nrmse(plain["pupil"], expected["pupil"]) > 2 * NRMSE  # the pupil did move


@pytest.mark.parametrize("n,side,batch", [(32, 5, 1), (64, 3, 4), (128, 3, 9)])
def test_gradient_descent_object_tv(fpm, n, side, batch):
    """GD with the object TV regulariser at every batch end
    (src/algorithms/gradient_descent.rs:643-651, regularization.rs:5-48)."""
    model, omodel, data, truth, gains = helpers.simulated(fpm, side, n, seed=31, photons=1e4)
    kw = dict(iterations=3, batch_size=batch, object_tv_weight=0.05, object_tv_epsilon=1e-6)
    algo = fpm.GradientDescent(iterations=3, batch_size=batch, object_tv=0.05, object_tv_epsilon=1e-6)
    result, expected = _run_both(fpm, algo, "gd", kw, model, omodel, data, gains=gains)
    assert oracle.complex_nrmse(expected["object"], result.object) <= NRMSE
    _objective_close([t[1] for t in result.trace], expected["objectives"])
    plain = oracle.run(oracle.Problem(omodel, data, gains=gains), "gd", iterations=3, batch_size=batch)
    assert oracle.complex_nrmse(plain["object"], expected["object"]) > 10 * NRMSE  # the regulariser acted


@pytest.mark.parametrize("n,side,batch", [(32, 5, 1), (64, 3, 4)])
def test_gradient_descent_pupil_smoothing(fpm, n, side, batch):
    """GD pupil recovery with quadratic pupil smoothing before the support
    (src/algorithms/gradient_descent.rs:653-663, regularization.rs:50-80)."""
    model, omodel, data, truth, gains = helpers.simulated(fpm, side, n, seed=32, photons=1e4, pupil_seed=5)
    kw = dict(iterations=3, batch_size=batch, recover_pupil=True, pupil_step=0.05, pupil_smoothing_weight=0.5)
    algo = fpm.GradientDescent(iterations=3, batch_size=batch, recover_pupil=True, pupil_step=0.05,
                               pupil_smoothing=0.5)
    result, expected = _run_both(fpm, algo, "gd", kw, model, omodel, data, gains=gains)
    assert oracle.complex_nrmse(expected["object"], result.object) <= NRMSE
    assert oracle.complex_nrmse(expected["pupil"], result.recovered_pupil) <= NRMSE
    assert np.all(result.recovered_pupil[model.pupil_support == 0] == 0)
    plain = oracle.run(oracle.Problem(omodel, data, gains=gains), "gd", iterations=3, batch_size=batch,
                       recover_pupil=True, pupil_step=0.05)
    assert oracle.complex_nrmse(plain["pupil"], expected["pupil"]) > 10 * NRMSE  # the smoothing acted


def test_regulariser_validation(fpm):
    model, omodel, data, truth, gains = helpers.simulated(fpm, 3, 32, seed=33)
    problem = fpm.ReconstructionProblem(data, model)
    for bad in (dict(object_tv=-1.0), dict(object_tv=0.1, object_tv_epsilon=0.0), dict(pupil_smoothing=0.1)):
        with pytest.raises(fpm.FpmError):
            fpm.GradientDescent(iterations=1, **bad).run(problem)
    with pytest.raises(fpm.UnsupportedError):
        fpm.GradientDescent(iterations=1, object_tv=0.1, loss_type="poisson_nll",
                            poisson_truncation_threshold=25.0).run(problem)


def test_empty_batch_zero_iterations_and_large_grid(fpm):
    """Edge cases: an empty batch, zero iterations (the measured-amplitude
    initial object, src/reconstruction/state.rs:280-355), and 64-point tiles
    on an exact 1024 x 1024 grid (crops far from the grid edges)."""
    assert fpm.run_batch(fpm.Mpie(iterations=2), []) == []
    model, omodel, data, truth, gains = helpers.simulated(fpm, 5, 32, seed=41, photons=1e4)
    result, expected = _run_both(fpm, fpm.AlternatingProjection(iterations=0), "ap", dict(iterations=0), model,
                                 omodel, data, gains=gains)
    assert result.trace == []
    assert oracle.complex_nrmse(expected["object"], result.object) <= 1e-6
    big, obig = helpers.planar_model(fpm, 5, 64, shape_policy=(1024, 1024))
    assert big.reconstruction_shape == (1024, 1024)
    obj = W.smooth_random_object((1024, 1024), 42)
    intensity = oracle.forward_stack(oracle.Problem(obig, None), oracle.object_spectrum(obj), workers=8)
    result, expected = _run_both(fpm, fpm.Mpie(iterations=2), "mpie", dict(iterations=2), big, obig, intensity)
    assert oracle.complex_nrmse(expected["object"], result.object) <= NRMSE
    _objective_close([t[1] for t in result.trace], expected["objectives"])


def test_ragged_batch_of_all_tile_sizes(fpm):
    """One batch mixing every tile size and LED count equals each tile's own run, bitwise."""
    specs = [(3, 32, 51), (5, 64, 52), (3, 128, 53), (3, 256, 54), (5, 32, 55)]
    problems = []
    for side, n, seed in specs:
        model, omodel, data, truth, gains = helpers.simulated(fpm, side, n, seed=seed, photons=1e4)
        problems.append(fpm.ReconstructionProblem(data, model))
    algo = fpm.Mpie(iterations=2)
    batch = fpm.run_batch(algo, problems)
    for p, got in zip(problems, batch):
        alone = algo.run(p)
        np.testing.assert_array_equal(alone.object_spectrum, got.object_spectrum)
