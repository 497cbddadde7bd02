"""Pins the FP64 oracle to the reference's own known-answer tests.

Every test restates a reference test with its tolerance: the cited file:line
is in hgrecco/fpm-rs. The reference publishes no numeric golden files for
this path; its known answers are these analytic properties and exact values.
"""

from __future__ import annotations

import math

import numpy as np
import pytest

import oracle
import workloads as W


@pytest.fixture(scope="module", autouse=True)
def _built(oracle_module):
    return oracle_module


def direct_model():
    """tests/common/mod.rs:49-81: 8x8 frames, 16x16 object, five integer shifts, unit pupil."""
    shifts = [(-3, 0), (0, -3), (0, 0), (0, 3), (3, 0)]  # (column, row)
    return dict(h=8, w=8, mh=16, mw=16,
                start_row=np.array([4 + r for c, r in shifts], np.int64),
                start_col=np.array([4 + c for c, r in shifts], np.int64),
                off_row=np.zeros(5), off_col=np.zeros(5),
                pupil=np.ones((8, 8), np.complex128), support=np.ones((8, 8), np.uint8),
                kx=np.array([float(c) for c, r in shifts]), ky=np.array([float(r) for c, r in shifts]))


def test_fft_forward_inverse_round_trip():
    # tests/forward_model_tests.rs:12-31
    index = np.arange(7 * 9)
    original = (index / 13.0 + 1j * (index % 5)).reshape(7, 9)
    back = oracle.fft2(oracle.fft2(original), inverse=True)
    assert np.abs(back - original).max() <= 1e-10


@pytest.mark.parametrize("shape", [(7, 9), (42, 42), (96, 96), (189, 189), (13, 17), (37, 1031),
                                   # power-of-two paths: even and odd exponents, groups of eight rows
                                   # with a ragged tail, and either axis a power of two alone
                                   (32, 32), (128, 128), (256, 256), (2, 512), (12, 64), (8, 96), (96, 8),
                                   (1, 16), (16, 1)])
def test_fft_matches_numpy_with_reference_normalisation(shape):
    # CpuBackend::fft2 (src/backend/cpu.rs:162-172): forward / N, inverse unscaled.
    rng = np.random.default_rng(1)
    values = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    assert np.abs(oracle.fft2(values) - np.fft.fft2(values) / values.size).max() <= 1e-13
    assert np.abs(oracle.fft2(values, inverse=True) - np.fft.ifft2(values) * values.size).max() <= 1e-9


def test_shift_conventions():
    # src/model/forward.rs:530-569: fftshift moves by floor(n/2), ifftshift by ceil(n/2).
    for shape in [(7, 9), (8, 8), (5, 6)]:
        a = np.arange(np.prod(shape)).reshape(shape) + 0j
        assert np.array_equal(oracle.fftshift(a), np.fft.fftshift(a))
        assert np.array_equal(oracle.ifftshift(a), np.fft.ifftshift(a))


def test_constant_object_has_constant_central_frame():
    # tests/forward_model_tests.rs:75-101: amplitude 2 -> intensity 4 everywhere.
    m = direct_model()
    spatial = np.full((16, 16), 2.0 + 0j)
    spectrum = oracle.fft2(spatial)
    centred = np.zeros_like(spectrum)
    for row in range(16):
        for col in range(16):
            centred[(row + 8) % 16, (col + 8) % 16] = spectrum[row, col]
    intensity = oracle.forward_stack(oracle.Problem(m, None), centred)
    assert np.all(np.abs(intensity[2] - 4.0) < 1e-10)


def test_patch_extraction_and_update_are_consistent():
    # tests/forward_model_tests.rs:103-114
    spectrum = np.zeros((16, 16), np.complex128)
    update = np.full((8, 8), 1.0 - 0.5j)
    out = oracle.insert_adjoint(spectrum, (4, 4), update, 1.0)
    patch = oracle.extract_patch(out, (4, 4), (8, 8))
    assert np.array_equal(patch, update)


def test_subpixel_patch_uses_bilinear_fourier_sampling():
    # tests/forward_model_tests.rs:116-152: offset (0.25, 0.5) on a linear ramp, 1e-12.
    rows, cols = np.indices((16, 16))
    spectrum = (1.0 + 2.0 * rows + 3.0 * cols) + 1j * (-rows + 0.5 * cols)
    patch = oracle.extract_patch(spectrum, (4, 4), (8, 8), (0.25, 0.5))
    r, c = np.indices((8, 8))
    sr, sc = 4.25 + r, 4.5 + c
    expected = (1.0 + 2.0 * sr + 3.0 * sc) + 1j * (-sr + 0.5 * sc)
    assert np.abs(patch - expected).max() <= 1e-12


@pytest.mark.parametrize("cycles", [1, 4, 8])
def test_bilinear_attenuation_law(cycles):
    # tests/forward_model_tests.rs:154-216: half-pixel interpolation of
    # exp(i 2 pi nu r / H) has relative RMS error 1 - cos(pi nu / H).
    shape = (32, 32)
    rows = np.indices(shape)[0]
    spectrum = np.exp(1j * 2 * math.pi * cycles * rows / shape[0])
    sampled = oracle.extract_patch(spectrum, (10, 10), (8, 8), (0.5, 0.0))
    ref_rows = 10 + np.indices((8, 8))[0] + 0.5
    reference = np.exp(1j * 2 * math.pi * cycles * ref_rows / shape[0])
    error = math.sqrt(np.mean(np.abs(sampled - reference) ** 2))
    assert abs(error - (1.0 - math.cos(math.pi * cycles / shape[0]))) <= 1e-12


def test_subpixel_insertion_is_the_exact_adjoint():
    # tests/forward_model_tests.rs:218-258, offset (-0.3, 0.4), 1e-12.
    idx = np.arange(256)
    spectrum = ((idx % 13) / 7.0 + 1j * ((idx % 17) / 11.0 - 0.5)).reshape(16, 16)
    k = np.arange(64)
    update = ((k % 7) / 5.0 - 0.4 + 1j * ((k % 11) / 9.0)).reshape(8, 8)
    extracted = oracle.extract_patch(spectrum, (4, 4), (8, 8), (-0.3, 0.4))
    adjoint = oracle.insert_adjoint(np.zeros((16, 16), np.complex128), (4, 4), update, 1.0, (-0.3, 0.4))
    left = np.sum(np.conj(extracted) * update)
    right = np.sum(np.conj(spectrum) * adjoint)
    assert abs(left - right) <= 1e-12 * 1.0 + 1e-12


def test_geometry_shift_sign_and_fractional_offsets():
    # tests/geometry_tests.rs:474-496: k = (1.25 dk, -0.5 dk) on (8, 8) -> (16, 16).
    optics = dict(W.OPTICS)
    pixel = optics["camera_pixel_size"] / optics["magnification"]
    dk = 2 * math.pi / (8 * pixel)
    m = oracle.compile_model(optics, [1.25 * dk], [-0.5 * dk], (8, 8), (16, 16))
    central = (16 - 8) // 2
    assert m["start_col"][0] > central
    assert m["start_row"][0] < central
    assert abs(m["off_col"][0] - 0.25) <= 1e-12
    assert abs(m["off_row"][0] - 0.5) <= 1e-12


def test_mpie_complex_recurrence_exact_values():
    # src/algorithms/common.rs:512-535 (bitwise).
    obj = np.array([3 + 2j, -1 + 0j])
    vel = np.array([1 + 0j, 0 - 2j])
    anc = np.array([1 + 1j, -2 + 0j])
    o, v, a = oracle.momentum_event(obj, vel, anc, 0.5, 0.25)
    assert v[0] == 2.5 + 1j and v[1] == 1 - 1j
    assert o[0] == 3.625 + 2.25j and o[1] == -0.75 - 0.25j
    assert np.array_equal(a, o)


def test_mpie_recurrence_rejects_non_finite_values():
    # src/algorithms/common.rs:537-555
    with pytest.raises(oracle.OracleError):
        oracle.momentum_event(np.array([np.inf + 0j]), np.zeros(1, complex), np.zeros(1, complex), 0.9, 0.9)


def test_next_smooth_multiplier():
    # next_smooth_multiplier (src/model/image_plane_fpm.rs:1176-1198).
    for minimum, expected in [(1, 1), (11, 12), (42, 42), (43, 45), (365, 375), (722, 729), (97, 98)]:
        assert oracle.next_smooth(minimum) == expected


@pytest.mark.parametrize("side,n,expected", [(3, 32, 42), (15, 256, 729), (13, 128, 336), (15, 32, 96),
                                             (15, 64, 189), (15, 128, 375)])
def test_config_reconstruction_shapes(side, n, expected):
    grid, ref = W.led_grid(side)
    kx, ky = oracle.planar_kvectors(W.OPTICS, grid, W.PITCH, ref, (0.0, 0.0, W.Z))
    m = oracle.compile_model(W.OPTICS, kx, ky, (n, n))
    assert (m["mh"], m["mw"]) == (expected, expected)
    fractional = np.sum((np.abs(m["off_row"]) > 1e-12) | (np.abs(m["off_col"]) > 1e-12))
    assert fractional == side * side - 1  # every LED but the centre one


def _direct_problem(seed=3):
    m = direct_model()
    rng = np.random.default_rng(seed)
    obj = 1.0 + 0.1 * rng.standard_normal((16, 16)) + 0.1j * rng.standard_normal((16, 16))
    data = oracle.forward_stack(oracle.Problem(m, None), oracle.object_spectrum(obj))
    return m, data


def test_alternating_projection_decreases_loss():
    # tests/reconstruction_tests.rs:66-101
    m, data = _direct_problem()
    out = oracle.run(oracle.Problem(m, data), "ap", iterations=5)
    assert out["objectives"][-1] < out["objectives"][0]


def test_mpie_without_feedback_equals_fpie_bitwise():
    # tests/reconstruction_tests.rs:655-691
    m, data = _direct_problem()
    fpie = oracle.run(oracle.Problem(m, data), "fpie", iterations=3, object_step=0.2, stability=0.05)
    mpie = oracle.run(oracle.Problem(m, data), "mpie", iterations=3, momentum_feedback=0.0, momentum_interval=2)
    assert np.array_equal(fpie["object_spectrum"], mpie["object_spectrum"])


def test_gradient_descent_decreases_loss():
    m, data = _direct_problem(5)
    out = oracle.run(oracle.Problem(m, data), "gd", iterations=5)
    assert out["objectives"][-1] < out["objectives"][0]


def test_epry_canonical_pupil_keeps_reference_energy():
    # Gauge canonicalisation matches the compiled pupil's supported energy
    # (src/algorithms/gauge.rs:158-240).
    m, data = _direct_problem(7)
    out = oracle.run(oracle.Problem(m, data * 1.3), "epry", iterations=3)
    energy = np.sum(np.abs(out["pupil"][m["support"] != 0]) ** 2)
    assert abs(energy - np.sum(m["support"])) <= 1e-9 * energy


def test_zero_weight_frames_are_ignored():
    # Frames with zero weight do not change the object (src/algorithms/common.rs:67-72).
    m, data = _direct_problem(9)
    w = np.ones(5)
    w[1] = 0.0
    corrupted = data.copy()
    corrupted[1] *= 7.0
    a = oracle.run(oracle.Problem(m, data, weights=w), "ap", iterations=2)
    b = oracle.run(oracle.Problem(m, corrupted, weights=w), "ap", iterations=2)
    assert np.array_equal(a["object_spectrum"], b["object_spectrum"])


def test_poisson_truncation_gate_includes_its_boundary():
    # src/algorithms/gradient_descent.rs:1389-1395
    assert oracle.truncation_accepts(4.0, 10.0, 3.0)
    assert not oracle.truncation_accepts(4.0, 10.000_001, 3.0)
    assert oracle.truncation_accepts(0.0, 0.0, 1.0)
    assert not oracle.truncation_accepts(0.0, 1.0, 1.0)


def test_poisson_truncation_requires_poisson_loss_and_is_inert_when_wide():
    # GradientDescent::validate (src/algorithms/gradient_descent.rs:319-331);
    # a threshold so large that every pixel passes leaves GD unchanged.
    m, data = _direct_problem(11)
    with pytest.raises(oracle.OracleError):
        oracle.run(oracle.Problem(m, data), "gd", iterations=1, poisson_truncation_threshold=25.0)
    plain = oracle.run(oracle.Problem(m, data), "gd", iterations=3, batch_size=5, loss_type="poisson_nll")
    wide = oracle.run(oracle.Problem(m, data), "gd", iterations=3, batch_size=5, loss_type="poisson_nll",
                      poisson_truncation_threshold=1e30)
    assert np.array_equal(plain["object_spectrum"], wide["object_spectrum"])
    tight = oracle.run(oracle.Problem(m, data * 1.7), "gd", iterations=3, batch_size=5, loss_type="poisson_nll",
                       poisson_truncation_threshold=0.05)
    loose = oracle.run(oracle.Problem(m, data * 1.7), "gd", iterations=3, batch_size=5, loss_type="poisson_nll")
    assert not np.array_equal(tight["object_spectrum"], loose["object_spectrum"])


def test_adaptive_ap_step_controller():
    # AdaptiveAlternatingProjection (src/algorithms/adaptive_alternating_projection.rs:245-307):
    # with progress_threshold 0 a pass that improves keeps the step; with a
    # threshold no pass can meet, the step halves every pass after the second
    # (floored at the minimum), so the run differs from AP at a fixed step.
    m, data = _direct_problem(13)
    ap = oracle.run(oracle.Problem(m, data), "ap", iterations=4)
    keep = oracle.run(oracle.Problem(m, data), "adaptive_ap", iterations=4, progress_threshold=0.0)
    assert np.array_equal(ap["object_spectrum"], keep["object_spectrum"])
    shrink = oracle.run(oracle.Problem(m, data), "adaptive_ap", iterations=4, progress_threshold=0.999,
                        minimum_object_step=0.3)
    assert not np.array_equal(ap["object_spectrum"], shrink["object_spectrum"])
    two = oracle.run(oracle.Problem(m, data), "adaptive_ap", iterations=2, progress_threshold=0.999)
    ap2 = oracle.run(oracle.Problem(m, data), "ap", iterations=2)
    assert np.array_equal(ap2["object_spectrum"], two["object_spectrum"])  # no comparison before pass 3
    with pytest.raises(oracle.OracleError):
        oracle.run(oracle.Problem(m, data), "adaptive_ap", iterations=2, reduction_factor=1.0)


def test_gd_pupil_recovery_moves_the_pupil_inside_its_support():
    # GradientDescent pupil recovery (src/algorithms/gradient_descent.rs:563-656):
    # the pupil changes, stays zero outside the support, and the gauge keeps
    # the compiled pupil's supported energy (src/algorithms/gauge.rs:158-240).
    m, data = _direct_problem(17)
    m = dict(m)
    support = np.ones((8, 8), np.uint8)
    support[0, :] = 0
    m["support"] = support
    m["pupil"] = m["pupil"] * support
    out = oracle.run(oracle.Problem(m, data * 1.2), "gd", iterations=3, batch_size=5, recover_pupil=True,
                     pupil_step=0.05)
    plain = oracle.run(oracle.Problem(m, data * 1.2), "gd", iterations=3, batch_size=5)
    assert not np.array_equal(out["pupil"], plain["pupil"])
    assert np.all(out["pupil"][support == 0] == 0)
    energy = np.sum(np.abs(out["pupil"][support != 0]) ** 2)
    assert abs(energy - np.sum(support)) <= 1e-9 * energy


def test_regulariser_known_answers(oracle_module):
    # apply_complex_tv_step / apply_quadratic_smoothing_step
    # (src/algorithms/regularization.rs:5-80) on a 1x2 array, closed form.
    a, b, w, eps = 1.0 + 0.5j, -0.25 + 2.0j, 0.3, 0.1
    d = b - a
    norm = np.sqrt(abs(d) ** 2 + eps ** 2)
    got = oracle_module.complex_tv_step(np.array([[a, b]]), w, eps)
    np.testing.assert_allclose(got[0], [a + w * d / norm, b - w * d / norm], rtol=0, atol=1e-15)
    got = oracle_module.quadratic_smoothing_step(np.array([[a, b]]), w)
    np.testing.assert_allclose(got[0], [a + 2 * w * d, b - 2 * w * d], rtol=0, atol=1e-15)
    # Zero weight is the identity; the single-column case has vertical terms only.
    x = np.array([[a], [b]])
    np.testing.assert_array_equal(oracle_module.complex_tv_step(x, 0.0, eps), x)
    got = oracle_module.complex_tv_step(x, w, eps)
    np.testing.assert_allclose(got[:, 0], [a + w * d / norm, b - w * d / norm], rtol=0, atol=1e-15)


def test_regularisers_reduce_variation_and_roughness(oracle_module):
    # tests/reconstruction_tests.rs:2513-2600: a checkerboard object and pupil.
    rows, cols = np.indices((16, 16))
    sign = np.where((rows + cols) % 2 == 0, 1.0, -1.0)
    obj = (1.0 + 0.15 * sign) * np.exp(1j * 0.2 * sign)

    def variation(v):
        return np.abs(np.diff(v, axis=1)).sum() + np.abs(np.diff(v, axis=0)).sum()

    assert variation(oracle_module.complex_tv_step(obj, 0.002, 1e-6)) < variation(obj)
    pupil = np.exp(1j * 0.35 * sign)
    assert variation(oracle_module.quadratic_smoothing_step(pupil, 0.02)) < variation(pupil)


def _direct_model():
    # tests/common/mod.rs:49-81: 8x8 detector, 16x16 grid, unit pupil, five
    # integer crops at (4 + row, 4 + column) for (column, row) shifts.
    shifts = [(-3, 0), (0, -3), (0, 0), (0, 3), (3, 0)]
    return dict(h=8, w=8, mh=16, mw=16, start_row=np.array([4 + r for c, r in shifts], np.int64),
                start_col=np.array([4 + c for c, r in shifts], np.int64), off_row=np.zeros(5), off_col=np.zeros(5),
                pupil=np.ones((8, 8), np.complex128), support=np.ones((8, 8), np.uint8))


def _direction(length, scale):
    i = np.arange(length)
    return scale * ((i % 13) / 13.0 - 0.5) + 1j * scale * ((i % 17) / 17.0 - 0.5)


@pytest.mark.parametrize("loss", ["amplitude_mse", "intensity_mse", "poisson_nll", "huber_amplitude"])
def test_gradient_descent_gradients_match_finite_differences(oracle_module, loss):
    # tests/reconstruction_tests.rs:2189-2300: object and pupil gradients of
    # one GD step against central differences of the masked frame loss, 2e-5.
    o = oracle_module
    model = _direct_model()
    rng = np.random.default_rng(4)
    truth = np.exp(1j * 0.3 * rng.standard_normal((16, 16))) * (0.8 + 0.2 * rng.random((16, 16)))
    data = o.forward_stack(o.Problem(model, None), o.object_spectrum(truth))
    mask = np.ones((8, 8), np.uint8)
    mask.ravel()[::5] = 0
    problem = o.Problem(model, data, masks=np.broadcast_to(mask, data.shape).copy())
    idx = np.arange(256).reshape(16, 16)
    start = truth * (0.78 + 0.03 * (idx % 7) / 7.0) * np.exp(1j * 0.08 * ((idx % 11) / 11.0 - 0.5))
    spectrum = o.object_spectrum(start)
    pupil = model["pupil"]
    frame, eps = 2, 1e-10
    after, pupil_after = o.gd_batch_step(problem, spectrum, pupil, [frame], object_step=1.0, loss_type=loss,
                                         recover_pupil=True, pupil_step=1.0, constrain_pupil=False)
    d_obj = _direction(256, 0.07).reshape(16, 16)
    d_pup = _direction(64, 0.05).reshape(8, 8)

    def check(gradient, direction, perturb):
        analytical = 2.0 * np.sum((np.conj(gradient) * direction).real)
        h = 1e-6
        numerical = (perturb(h) - perturb(-h)) / (2 * h)
        scale = max(abs(analytical), abs(numerical), 1e-10)
        assert abs(analytical - numerical) <= 2e-5 * scale, (loss, analytical, numerical)

    obj_den = max(np.max(np.abs(pupil) ** 2), eps) + eps
    check((spectrum - after) * obj_den, d_obj,
          lambda t: o.frame_loss(problem, spectrum + t * d_obj, pupil, frame, loss))
    patch = o.extract_patch(spectrum, (model["start_row"][frame], model["start_col"][frame]), (8, 8))
    pup_den = max(np.max(np.abs(patch) ** 2), eps) + eps
    check((pupil - pupil_after) * pup_den, d_pup,
          lambda t: o.frame_loss(problem, spectrum, pupil + t * d_pup, frame, loss))


def test_gradient_minibatch_is_the_mean_of_frame_gradients(oracle_module):
    # tests/reconstruction_tests.rs:1802-1854: a two-frame batch moves the
    # object by the mean of the two single-frame moves (1e-12).
    o = oracle_module
    model = _direct_model()
    rng = np.random.default_rng(5)
    truth = np.exp(1j * 0.3 * rng.standard_normal((16, 16)))
    data = o.forward_stack(o.Problem(model, None), o.object_spectrum(truth))
    problem = o.Problem(model, data)
    start = o.object_spectrum(truth * 0.9)
    pupil = model["pupil"]
    firsts = [o.gd_batch_step(problem, start, pupil, [f], object_step=0.3)[0] for f in (0, 1)]
    batched = o.gd_batch_step(problem, start, pupil, [0, 1], object_step=0.3)[0]
    expected = start + ((firsts[0] - start) + (firsts[1] - start)) / 2.0
    np.testing.assert_allclose(batched, expected, rtol=0, atol=1e-12)


@pytest.mark.parametrize("loss", ["amplitude_mse", "intensity_mse", "poisson_nll", "huber_amplitude"])
def test_illumination_gradients_match_direct_loss_differences(oracle_module, loss):
    # tests/reconstruction_tests.rs:2300-2374: the source-offset gradient of
    # one GD step on frame 2 (every sixth pixel masked, a perturbed start)
    # against central differences of the masked frame loss at offsets +-d on
    # each axis, 5e-3 relative.
    o = oracle_module
    model = _direct_model()
    rng = np.random.default_rng(9)
    truth = np.exp(1j * 0.3 * rng.standard_normal((16, 16))) * (0.8 + 0.2 * rng.random((16, 16)))
    data = o.forward_stack(o.Problem(model, None), o.object_spectrum(truth))
    mask = (np.arange(64) % 6 != 1).astype(np.uint8).reshape(8, 8)
    masks = np.broadcast_to(mask, data.shape).copy()
    problem = o.Problem(model, data, masks=masks)
    idx = np.arange(256).reshape(16, 16)
    spectrum = o.object_spectrum(truth * 0.82 * np.exp(1j * 0.04 * (idx % 9) / 9.0))
    pupil = model["pupil"]
    frame, d = 2, 1e-4
    _, _, gradient = o.gd_batch_step(problem, spectrum, pupil, [frame], illumination_gradient=True,
                                     object_step=1e-12, loss_type=loss, recover_illumination=True,
                                     illumination_step=1e-12, illumination_finite_difference=d)

    def shifted_loss(drow, dcol):
        m = dict(model, off_row=model["off_row"].copy(), off_col=model["off_col"].copy())
        m["off_row"][frame] += drow
        m["off_col"][frame] += dcol
        return o.frame_loss(o.Problem(m, data, masks=masks), spectrum, pupil, frame, loss)

    for axis, (drow, dcol) in enumerate([(d, 0.0), (0.0, d)]):
        numerical = (shifted_loss(drow, dcol) - shifted_loss(-drow, -dcol)) / (2 * d)
        analytical = gradient[frame, axis]
        scale = max(abs(analytical), abs(numerical), 1e-10)
        assert abs(analytical - numerical) <= 5e-3 * scale, (loss, axis, analytical, numerical)
    assert np.all(gradient[[0, 1, 3, 4]] == 0.0)


def test_illumination_update_honours_bounds_and_the_grid(oracle_module):
    # GradientDescent::apply_illumination_update (src/algorithms/
    # gradient_descent.rs:1044-1089): each step is clamped to the correction
    # bound and kept only while the corrected crop stays inside the grid
    # (CropIndices::validate_subpixel_inside, src/model/crop.rs:105-113).
    o = oracle_module
    model = _direct_model()
    rng = np.random.default_rng(10)
    truth = np.exp(1j * 0.4 * rng.standard_normal((16, 16))) * (0.7 + 0.3 * rng.random((16, 16)))
    shifted = dict(model, off_row=model["off_row"].copy(), off_col=model["off_col"].copy())
    shifted["off_row"][1], shifted["off_col"][1] = 0.3, -0.2
    data = o.forward_stack(o.Problem(shifted, None), o.object_spectrum(truth))
    out = o.run(o.Problem(model, data), "gd", iterations=20, recover_illumination=True, illumination_step=0.5,
                illumination_bounds=0.1)
    corr = out["illumination_corrections"]
    # The displaced source saturates at the bound on the side of its displacement.
    np.testing.assert_array_equal(corr[1], [0.1, -0.1])
    assert np.all(np.abs(corr) <= 0.1)
    # Crops touching the grid edge (rows 0 and 8, columns 0 and 8 of a
    # 16-point grid with 8-point frames) only move inward.
    edge = dict(model, start_row=np.array([0, 4, 4, 4, 8]), start_col=np.array([4, 0, 4, 8, 4]))
    data = o.forward_stack(o.Problem(edge, None), o.object_spectrum(truth)) * 1.1
    corr = o.run(o.Problem(edge, data), "gd", iterations=20, recover_illumination=True, illumination_step=1.0,
                 illumination_bounds=0.5)["illumination_corrections"]
    assert corr[0, 0] >= 0.0 and corr[4, 0] <= 0.0 and corr[1, 1] >= 0.0 and corr[3, 1] <= 0.0, corr
    assert np.abs(corr).max() > 0.05


def test_mpie_cadence_is_independent_of_batch_partitioning(oracle_module):
    # tests/reconstruction_tests.rs:693-731: bitwise equal spectra and traces.
    o = oracle_module
    model = _direct_model()
    truth = np.exp(1j * 0.3 * np.random.default_rng(6).standard_normal((16, 16)))
    data = o.forward_stack(o.Problem(model, None), o.object_spectrum(truth))
    problem = o.Problem(model, data)
    single = o.run(problem, "mpie", iterations=4, momentum_interval=3, batch_size=1)
    grouped = o.run(problem, "mpie", iterations=4, momentum_interval=3, batch_size=5)
    np.testing.assert_array_equal(single["object_spectrum"], grouped["object_spectrum"])
    np.testing.assert_array_equal(single["objectives"], grouped["objectives"])


def test_gauge_keeps_predictions_and_is_idempotent(oracle_module):
    # src/algorithms/gauge.rs:435-496: integer crops, a perturbed state;
    # canonicalisation leaves every prediction unchanged (2e-12), and a second
    # pass changes nothing; invalid fields are numerical errors.
    o = oracle_module
    model = _direct_model()
    rng = np.random.default_rng(8)
    truth = np.exp(1j * 0.3 * rng.standard_normal((16, 16)))
    data = o.forward_stack(o.Problem(model, None), o.object_spectrum(truth))
    problem = o.Problem(model, data)
    rows, cols = np.indices((8, 8))
    pupil = 1.7 * np.exp(1j * (0.4 + 0.17 * rows - 0.23 * cols))
    spectrum = o.object_spectrum(truth) * 0.6 * np.exp(-0.9j)
    before = o.forward_stack(o.Problem(dict(model, pupil=pupil), None), spectrum)
    canon_s, canon_p = o.canonicalize(problem, spectrum, pupil)
    after = o.forward_stack(o.Problem(dict(model, pupil=canon_p), None), canon_s)
    assert np.max(np.abs(after - before)) <= 2e-12 * np.max(np.abs(before))
    again_s, again_p = o.canonicalize(problem, canon_s, canon_p)
    np.testing.assert_array_equal(again_s, canon_s)
    np.testing.assert_array_equal(again_p, canon_p)
    with pytest.raises(o.OracleError):
        o.canonicalize(problem, spectrum, np.zeros_like(pupil))
    bad = spectrum.copy()
    bad[0, 0] = np.nan
    with pytest.raises(o.OracleError):
        o.canonicalize(problem, bad, pupil)


def _mixed_test_pattern(shape):
    # SyntheticObject::mixed_test_pattern (src/simulation/synthetic_object.rs:
    # 275-298): an absorbing bar and disc on a Gaussian phase bump plus a sine.
    rows, cols = np.indices(shape, dtype=np.float64)
    y, x = rows - (shape[0] - 1) / 2.0, cols - (shape[1] - 1) / 2.0
    scale = float(min(shape))
    radius = np.hypot(x, y)
    absorbing = ((np.abs(x) < 0.12 * scale) & (np.abs(y) < 0.35 * scale)) | (radius < 0.12 * scale)
    amplitude = np.where(absorbing, 0.45, 1.0)
    phase = 0.8 * np.exp(-radius * radius / (0.08 * scale * scale)) + 0.25 * np.sin(2 * np.pi * x / scale)
    return amplitude * np.exp(1j * phase)


def _offset_problem(o, offsets):
    model = _direct_model()
    truth = _mixed_test_pattern((16, 16))
    true_model = dict(model, off_row=np.array([r for r, c in offsets]), off_col=np.array([c for r, c in offsets]))
    data = o.forward_stack(o.Problem(true_model, None), o.object_spectrum(truth))
    return model, truth, o.Problem(model, data)


def test_gradient_recovers_known_source_offsets_with_fixed_object(oracle_module):
    # tests/reconstruction_tests.rs:1322-1371: from the true object with a
    # negligible object step, 8 full-batch steps halve the offset error.
    o = oracle_module
    offsets = [(0.20, -0.15), (-0.18, 0.22), (0.16, 0.12), (-0.20, -0.14), (0.14, -0.20)]
    model, truth, problem = _offset_problem(o, offsets)
    spectrum, pupil = o.object_spectrum(truth), model["pupil"]
    corrections = np.zeros((5, 2))
    for _ in range(8):
        spectrum, pupil = o.gd_batch_step(problem, spectrum, pupil, range(5), corrections=corrections,
                                          object_step=1e-10, recover_illumination=True, illumination_step=0.5,
                                          illumination_finite_difference=0.02, illumination_bounds=0.75)
    initial = sum(r * r + c * c for r, c in offsets)
    final = float(np.sum((corrections - np.array(offsets)) ** 2))
    assert final < 0.5 * initial, (initial, final, corrections)


def test_joint_illumination_calibration_reduces_model_mismatch(oracle_module):
    # tests/reconstruction_tests.rs:1373-1427: every source displaced by
    # (0.22, -0.18); full-batch GD for 20 iterations with recovery reaches a
    # lower objective than without, and the offset error falls.
    o = oracle_module
    offsets = [(0.22, -0.18)] * 5
    model, truth, problem = _offset_problem(o, offsets)
    kw = dict(iterations=20, object_step=0.3, batch_size=5)
    plain = o.run(problem, "gd", **kw)
    calibrated = o.run(problem, "gd", recover_illumination=True, illumination_step=0.05,
                       illumination_finite_difference=0.02, illumination_bounds=0.75, **kw)
    assert calibrated["objectives"][-1] < plain["objectives"][-1]
    initial = sum(r * r + c * c for r, c in offsets)
    final = float(np.sum((calibrated["illumination_corrections"] - np.array(offsets)) ** 2))
    assert final < initial, (initial, final)


def _gain_error(reference, candidate):
    # compare_frame_gains (src/metrics/model.rs:130-161): relative L2 error
    # after one global positive scale.
    reference, candidate = np.asarray(reference), np.asarray(candidate)
    alignment = np.dot(candidate, reference) / max(np.dot(candidate, candidate), np.finfo(float).eps)
    return math.sqrt(np.sum((alignment * candidate - reference) ** 2) / max(np.dot(reference, reference),
                                                                          np.finfo(float).eps))


def test_epry_recovers_relative_frame_gain_mismatch(oracle_module):
    # tests/reconstruction_tests.rs:3037-3079: a constant object (amplitude 2)
    # seen with frame gains (0.5, 1, 1.5, 2, 0.75); two EPRY passes with gain
    # recovery (step 1) cut the scale-aligned gain error tenfold.
    o = oracle_module
    model = _direct_model()
    true_gains = np.array([0.5, 1.0, 1.5, 2.0, 0.75])
    data = o.forward_stack(o.Problem(model, None, gains=true_gains), o.object_spectrum(np.full((16, 16), 2.0 + 0j)))
    out = o.run(o.Problem(model, data), "epry", iterations=2, object_step=1e-6, recover_pupil=False,
                recover_gains=True, gain_step=1.0)
    mean = true_gains.mean()
    initial = math.sqrt(np.sum((mean - true_gains) ** 2) / np.sum(true_gains ** 2))
    assert _gain_error(true_gains, out["frame_gains"]) < 0.1 * initial


def test_epry_recovers_relative_per_frame_background(oracle_module):
    # tests/reconstruction_tests.rs:3081-3123: per-frame constant backgrounds
    # (0, 1, 2, 3, 0.5); one EPRY pass with background recovery (step 1,
    # bounds [-10, 10]) recovers them up to a common offset, 1e-8.
    o = oracle_module
    model = _direct_model()
    true_bg = np.array([0.0, 1.0, 2.0, 3.0, 0.5])
    background = np.repeat(true_bg, 64).reshape(5, 8, 8)
    data = o.forward_stack(o.Problem(model, None, background=background),
                           o.object_spectrum(np.full((16, 16), 2.0 + 0j)))
    out = o.run(o.Problem(model, data), "epry", iterations=1, object_step=1e-6, recover_pupil=False,
                recover_background=True, background_step=1.0, background_min=-10.0, background_max=10.0)
    means = out["background"].reshape(5, -1).mean(axis=1)
    np.testing.assert_allclose(means - means.mean(), true_bg - true_bg.mean(), rtol=0, atol=1e-8)


def _ideal_direct(o, obj=None, **model_kw):
    model = dict(_direct_model(), **model_kw)
    obj = _mixed_test_pattern((16, 16)) if obj is None else obj
    return model, o.forward_stack(o.Problem(model, None), o.object_spectrum(obj))


def test_fpie_loss_decreases_on_noiseless_data(oracle_module):
    # tests/reconstruction_tests.rs:638-653 (the reference's test object is a
    # resolution target; the mixed test pattern stands in).
    o = oracle_module
    model, data = _ideal_direct(o)
    out = o.run(o.Problem(model, data), "fpie", iterations=8)
    assert out["objectives"][-1] < out["objectives"][0]


def test_projection_and_gradient_support_subpixel_crops(oracle_module):
    # tests/reconstruction_tests.rs:1284-1321: fractional offsets on every
    # source; AP (step 0.4) and GD (step 0.3, batch 2) both lower the loss.
    o = oracle_module
    offsets = [(-0.2, 0.3), (0.25, -0.35), (0.1, 0.2), (-0.3, -0.15), (0.2, 0.25)]
    model, data = _ideal_direct(o, off_row=np.array([r for r, c in offsets]),
                                off_col=np.array([c for r, c in offsets]))
    for name, kw in (("ap", dict(object_step=0.4)), ("gd", dict(object_step=0.3, batch_size=2))):
        out = o.run(o.Problem(model, data), name, iterations=8, **kw)
        assert out["objectives"][-1] < out["objectives"][0], name


@pytest.mark.parametrize("loss,step", [("intensity_mse", 0.05), ("poisson_nll", 0.2), ("huber_amplitude", 0.5)])
def test_gradient_solver_supports_configurable_losses(oracle_module, loss, step):
    # tests/reconstruction_tests.rs:2030-2059
    o = oracle_module
    model, data = _ideal_direct(o)
    out = o.run(o.Problem(model, data), "gd", iterations=8, object_step=step, loss_type=loss)
    assert out["objectives"][-1] < out["objectives"][0], loss


def test_gradient_loss_is_invariant_to_known_linear_camera_response(oracle_module):
    # tests/reconstruction_tests.rs:2602-2652: counts = g I + b with the gain
    # and offset compiled into the model leave the GD objectives (1e-12) and
    # the object spectrum (1e-11) unchanged.
    o = oracle_module
    model, data = _ideal_direct(o)
    gain, offset = 60.0, 13.0
    ideal = o.run(o.Problem(model, data), "gd", iterations=4)
    camera = o.run(o.Problem(model, gain * data + offset, gains=np.full(5, gain),
                             background=np.full((5, 8, 8), offset)), "gd", iterations=4)
    np.testing.assert_allclose(camera["objectives"], ideal["objectives"], rtol=0, atol=1e-12)
    np.testing.assert_allclose(camera["object_spectrum"], ideal["object_spectrum"], rtol=0, atol=1e-11)


def test_initialization_undoes_known_frame_gain_and_background(oracle_module):
    # tests/reconstruction_tests.rs:2713-2735: gain 4 and background 9 on a
    # constant amplitude-2 object; zero AP iterations return amplitude 2.
    o = oracle_module
    model = _direct_model()
    gains, background = np.full(5, 4.0), np.full((5, 8, 8), 9.0)
    data = o.forward_stack(o.Problem(model, None, gains=gains, background=background),
                           o.object_spectrum(np.full((16, 16), 2.0 + 0j)))
    out = o.run(o.Problem(model, data, gains=gains, background=background), "ap", iterations=0)
    assert np.abs(np.abs(out["object"]) - 2.0).max() <= 1e-10


def test_masked_pixels_do_not_affect_reconstruction(oracle_module):
    # tests/reconstruction_tests.rs:2820-2851: a masked pixel set to 1e12 in
    # every frame leaves three AP iterations bit for bit unchanged.
    o = oracle_module
    model, data = _ideal_direct(o)
    masks = np.ones(data.shape, np.uint8)
    masks[:, 0, 0] = 0
    corrupted = data.copy()
    corrupted[:, 0, 0] = 1.0e12
    clean = o.run(o.Problem(model, data, masks=masks), "ap", iterations=3)
    dirty = o.run(o.Problem(model, corrupted, masks=masks), "ap", iterations=3)
    np.testing.assert_array_equal(clean["object_spectrum"], dirty["object_spectrum"])


def test_forward_stack_is_independent_of_worker_count(oracle_module):
    # tests/forward_model_tests.rs:273-331 (single-source model): the
    # threaded forward stack equals the serial one bit for bit.
    o = oracle_module
    model = _direct_model()
    idx = np.arange(256)
    spectrum = ((idx % 17) / 13.0 + 1j * (idx % 11) / 9.0).reshape(16, 16)
    serial = o.forward_stack(o.Problem(model, None), spectrum, workers=1)
    np.testing.assert_array_equal(o.forward_stack(o.Problem(model, None), spectrum, workers=3), serial)


def test_amplitude_gradient_loss_decreases_on_single_source_data(oracle_module):
    # tests/reconstruction_tests.rs:1263-1281
    o = oracle_module
    model, data = _ideal_direct(o)
    out = o.run(o.Problem(model, data), "gd", iterations=8, object_step=0.5)
    assert out["objectives"][-1] < out["objectives"][0]


def test_truncated_poisson_gradient_rejects_outliers_and_improves_object_error(oracle_module):
    # tests/reconstruction_tests.rs:2061-2137: each frame's brightest pixel
    # scaled by 100; from a perturbed truth, 8 full-batch Poisson GD steps
    # (0.08) with the truncation gate at 25 end closer to the truth than
    # without it.
    o = oracle_module
    truth = _mixed_test_pattern((16, 16))
    model, data = _ideal_direct(o, truth)
    flat = data.reshape(5, -1)
    flat[np.arange(5), flat.argmax(axis=1)] *= 100.0
    idx = np.arange(256).reshape(16, 16)
    start = o.object_spectrum(truth * 0.82 * np.exp(1j * 0.12 * (idx % 13) / 13.0))
    kw = dict(iterations=8, object_step=0.08, batch_size=5, loss_type="poisson_nll", initial_spectrum=start)
    plain = o.run(o.Problem(model, data), "gd", **kw)
    gated = o.run(o.Problem(model, data), "gd", poisson_truncation_threshold=25.0, **kw)
    assert o.complex_nrmse(truth, gated["object"]) < o.complex_nrmse(truth, plain["object"])


def test_adaptive_projection_matches_fixed_step_until_feedback_has_two_objectives(oracle_module):
    # tests/reconstruction_tests.rs:103-125: two passes at 0.7 equal AP at
    # 0.7 bitwise, with the step trace (0.7, 0.7).
    o = oracle_module
    model, data = _ideal_direct(o)
    fixed = o.run(o.Problem(model, data), "ap", iterations=2, object_step=0.7)
    adaptive = o.run(o.Problem(model, data), "adaptive_ap", iterations=2, object_step=0.7)
    np.testing.assert_array_equal(adaptive["object_spectrum"], fixed["object_spectrum"])
    assert list(adaptive["object_steps"]) == [0.7, 0.7]


def test_adaptive_projection_reduces_the_step_to_its_floor(oracle_module):
    # tests/reconstruction_tests.rs:127-149: threshold 1 - eps, factor 0.5,
    # floor 0.2: steps (1, 1, 0.5, 0.25, 0.2, 0.2).
    o = oracle_module
    model, data = _ideal_direct(o)
    out = o.run(o.Problem(model, data), "adaptive_ap", iterations=6, progress_threshold=1.0 - np.finfo(float).eps,
                reduction_factor=0.5, minimum_object_step=0.2)
    assert list(out["object_steps"]) == [1.0, 1.0, 0.5, 0.25, 0.2, 0.2]


def test_mpie_accelerates_the_same_rpie_base_on_strong_phase_data(oracle_module):
    # tests/reconstruction_tests.rs:991-1050 on noiseless_mixed_fpm
    # (src/simulation/presets.rs:23-96: 3x3 LEDs, 4 mm pitch, z = -90 mm,
    # 32x32 frames, exact 64x64 grid) with the mixed pattern's phase x4: at
    # an equal frame-update budget mPIE (interval 10, friction and feedback
    # 0.7) ends below 0.95 x FPIE's objective and reaches 5.4e-5 first.
    o = oracle_module
    kx, ky = o.planar_kvectors(W.OPTICS, (3, 3), W.PITCH, (1.0, 1.0), (0.0, 0.0, W.Z))
    model = o.compile_model(W.OPTICS, kx, ky, (32, 32), (64, 64))
    base = _mixed_test_pattern((64, 64))
    strong = np.abs(base) * np.exp(4j * np.angle(base))
    data = o.forward_stack(o.Problem(model, None), o.object_spectrum(strong))
    fpie = o.run(o.Problem(model, data), "fpie", iterations=20, object_step=0.2, stability=0.05)["objectives"]
    mpie = o.run(o.Problem(model, data), "mpie", iterations=20, momentum_interval=10, momentum_friction=0.7,
                 momentum_feedback=0.7)["objectives"]
    assert mpie[-1] < 0.95 * fpie[-1], (fpie[-1], mpie[-1])
    target = 5.4e-5
    reached = [next((i for i, v in enumerate(t) if v < target), None) for t in (mpie, fpie)]
    assert reached[0] is not None and (reached[1] is None or reached[0] < reached[1]), reached


def _pupil_phase_rmse(recovered, truth, support):
    # pupil_phase_rmse (tests/reconstruction_tests.rs:3128-3149): phase RMSE
    # on the support after removing the global phase.
    inside = support != 0
    correction = np.exp(-1j * np.angle(np.sum(recovered[inside] * np.conj(truth[inside]))))
    diff = np.mod(np.angle(recovered[inside] * correction) - np.angle(truth[inside]) + np.pi, 2 * np.pi) - np.pi
    return math.sqrt(np.mean(diff * diff))


def test_epry_reduces_known_pupil_phase_error(oracle_module):
    # tests/reconstruction_tests.rs:2922-3010: data through a pupil with
    # -24 um defocus and astigmatism 0.2 (3x3 LEDs, 16x16 frames, exact
    # 32x32 grid, phase disk radius 8 and 0.9 rad); 40 EPRY passes (pupil
    # step 0.05) from the unaberrated pupil lower the pupil phase error.
    o = oracle_module
    kx, ky = o.planar_kvectors(W.OPTICS, (3, 3), W.PITCH, (1.0, 1.0), (0.0, 0.0, W.Z))
    assumed = o.compile_model(W.OPTICS, kx, ky, (16, 16), (32, 32))
    true_optics = dict(W.OPTICS, defocus_distance=-24e-6, pupil_aberration=dict(astigmatism=0.2))
    true = o.compile_model(true_optics, kx, ky, (16, 16), (32, 32))
    rows, cols = np.indices((32, 32))
    disk = np.hypot(rows - 15.5, cols - 15.5) <= 8.0
    obj = np.exp(1j * np.where(disk, 0.9, 0.0))  # SyntheticObject::phase_disk (synthetic_object.rs:156-180)
    data = o.forward_stack(o.Problem(true, None), o.object_spectrum(obj))
    out = o.run(o.Problem(assumed, data), "epry", iterations=40, pupil_step=0.05)
    initial = _pupil_phase_rmse(assumed["pupil"], true["pupil"], true["support"])
    recovered = _pupil_phase_rmse(out["pupil"], true["pupil"], true["support"])
    assert recovered < initial, (initial, recovered)
