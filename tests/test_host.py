"""Host-side checks that need no GPU: the C ABI library, model compilation
against the oracle (integer crop origins bit-exact), validation and error
mapping, and unsupported options failing before any device work."""

from __future__ import annotations

import ctypes as C
import math
import os
import re
from fractions import Fraction

import numpy as np
import pytest

import oracle
import workloads as W

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def fpm(native_library, oracle_module):
    import fpm_rs

    return fpm_rs


def _declared_symbols():
    text = open(os.path.join(ROOT, "include", "fpm_gpu.h")).read()
    return sorted(set(re.findall(r"^(?:int32_t|const char \*)\s*(fpm_\w+)\(", text, flags=re.M)))


def test_library_exports_every_declared_symbol(native_library):
    lib = C.CDLL(native_library)
    names = _declared_symbols()
    assert "fpm_run" in names and "fpm_problem_create" in names and len(names) >= 14
    for name in names:
        assert hasattr(lib, name), name


@pytest.mark.parametrize("side,n", [(3, 32), (15, 256), (13, 128), (15, 64), (9, 128), (5, 64)])
@pytest.mark.parametrize("policy", ["smooth", "minimum", "power_of_two"])
def test_compile_matches_oracle_bit_exact(fpm, side, n, policy):
    optics = fpm.Optics(**W.OPTICS)
    grid, ref = W.led_grid(side)
    geometry = fpm.PlanarLEDArray(grid, W.PITCH, ref, fpm.ArrayPose.from_translation((0.0, 0.0, W.Z)))
    model = fpm.compile_model(optics, fpm.Illumination(geometry), (n, n), policy)
    kx, ky = oracle.planar_kvectors(W.OPTICS, grid, W.PITCH, ref, (0.0, 0.0, W.Z))
    om = oracle.compile_model(W.OPTICS, kx, ky, (n, n), policy)
    assert model.reconstruction_shape == (om["mh"], om["mw"])
    assert np.array_equal(model.crop_origins[:, 0], om["start_row"])
    assert np.array_equal(model.crop_origins[:, 1], om["start_col"])
    assert np.array_equal(model.subpixel_offsets[:, 0], om["off_row"])
    assert np.array_equal(model.subpixel_offsets[:, 1], om["off_col"])
    assert np.array_equal(model.pupil_support, om["support"])
    assert np.array_equal(model.pupil, om["pupil"])
    assert np.array_equal(model.k_vectors[:, 0], kx) and np.array_equal(model.k_vectors[:, 1], ky)


def test_compile_with_defocus_aberration_and_rotation(fpm):
    ab = fpm.PupilAberration(astigmatism=0.3, coma=-0.2, spherical=0.1, edge_apodization=0.5)
    optics = fpm.Optics(**W.OPTICS, defocus_distance=5e-6, pupil_aberration=ab)
    pose = fpm.ArrayPose.from_translation_and_extrinsic_xyz_degrees((1e-3, -2e-3, -85e-3), (2.0, -1.0, 15.0))
    geometry = fpm.PlanarLEDArray((5, 7), (4e-3, 3.5e-3), (3.2, 1.7), pose)
    model = fpm.compile_model(optics, fpm.Illumination(geometry), (64, 64))
    odict = dict(W.OPTICS, defocus_distance=5e-6,
                 pupil_aberration=dict(astigmatism=0.3, coma=-0.2, spherical=0.1, edge_apodization=0.5))
    kx, ky = oracle.planar_kvectors(odict, (5, 7), (4e-3, 3.5e-3), (3.2, 1.7), (1e-3, -2e-3, -85e-3),
                                    tuple(np.radians([2.0, -1.0, 15.0])))
    om = oracle.compile_model(odict, kx, ky, (64, 64))
    assert np.array_equal(model.crop_origins[:, 0], om["start_row"])
    assert np.array_equal(model.crop_origins[:, 1], om["start_col"])
    assert np.abs(model.pupil - om["pupil"]).max() <= 1e-15


def test_exact_shape_validation(fpm):
    optics = fpm.Optics(**W.OPTICS)
    grid, ref = W.led_grid(3)
    geometry = fpm.PlanarLEDArray(grid, W.PITCH, ref, fpm.ArrayPose.from_translation((0.0, 0.0, W.Z)))
    with pytest.raises(fpm.InvalidShapeError):
        fpm.compile_model(optics, fpm.Illumination(geometry), (32, 32), (40, 40))
    with pytest.raises(fpm.InvalidShapeError):
        fpm.compile_model(optics, fpm.Illumination(geometry), (32, 32), (48, 50))
    assert fpm.suggest_reconstruction_shape(optics, fpm.Illumination(geometry), (32, 32)) == (42, 42)


def test_optics_validation(fpm):
    with pytest.raises(fpm.InvalidParameterError):
        fpm.Optics(532e-9, 0.1, 4.0, -6.5e-6)
    with pytest.raises(fpm.InvalidParameterError):
        fpm.Optics(532e-9, 0.5, 1.0, 6.5e-6)  # coherent sampling violated
    with pytest.raises(fpm.InvalidParameterError):
        fpm.Optics(532e-9, 1.2, 40.0, 6.5e-6)  # NA above the medium index


def test_coherent_sampling_is_strict_at_the_nyquist_boundary(fpm):
    # tests/geometry_tests.rs:26-65: pitch 4 / 2 equals 1 / (2 * 0.25) exactly;
    # the boundary itself is refused with the reference's wording, one ulp
    # below passes and one ulp above is refused.
    assert abs(fpm.Optics(532e-9, 0.1, 4.0, 6.5e-6).object_pixel_size - 1.625e-6) <= 1e-18
    with pytest.raises(fpm.InvalidParameterError) as info:
        fpm.Optics(1.0, 0.25, 2.0, 4.0)
    message = str(info.value)
    assert "strictly less" in message and "camera_pixel_size / magnification" in message
    assert "wavelength_vacuum_m / (2 * objective_na)" in message
    fpm.Optics(1.0, 0.25, 2.0, math.nextafter(4.0, 0.0))
    with pytest.raises(fpm.InvalidParameterError):
        fpm.Optics(1.0, 0.25, 2.0, math.nextafter(4.0, 5.0))


def test_measurement_and_problem_validation(fpm):
    model = fpm.compile_model(fpm.Optics(**W.OPTICS), fpm.Illumination(fpm.PlanarLEDArray(
        (3, 3), W.PITCH, (1.0, 1.0), fpm.ArrayPose.from_translation((0.0, 0.0, W.Z)))), (32, 32))
    data = np.ones((9, 32, 32))
    bad = data.copy()
    bad[0, 0, 0] = np.nan
    with pytest.raises(fpm.InvalidMeasurementsError):
        fpm.MeasurementStack(bad)
    with pytest.raises(fpm.InvalidMeasurementsError):
        fpm.MeasurementStack(data, frame_weights=[-1.0] + [1.0] * 8)
    with pytest.raises(fpm.InvalidModelError):
        fpm.ReconstructionProblem(np.ones((8, 32, 32)), model)
    with pytest.raises(fpm.InvalidShapeError):
        fpm.ReconstructionProblem(np.ones((9, 16, 16)), model)
    with pytest.raises(fpm.InvalidMeasurementsError):
        fpm.ReconstructionProblem(data, model, frame_weights=[0.0] * 9)
    masks = np.ones((9, 32, 32), np.uint8)
    masks[4] = 0
    with pytest.raises(fpm.InvalidMeasurementsError):
        fpm.ReconstructionProblem(data, model, masks=masks)


def test_unsupported_options_fail_before_device_work(fpm):
    model = fpm.compile_model(fpm.Optics(**W.OPTICS), fpm.Illumination(fpm.PlanarLEDArray(
        (3, 3), W.PITCH, (1.0, 1.0), fpm.ArrayPose.from_translation((0.0, 0.0, W.Z)))), (32, 32))
    problem = fpm.ReconstructionProblem(np.ones((9, 32, 32)), model)
    with pytest.raises(fpm.UnsupportedError):
        fpm.AlternatingProjection(iterations=1).run(problem, schedule="random")
    with pytest.raises(ValueError):
        fpm.AlternatingProjection(iterations=1).run(problem, schedule="spiral")
    # python/src/reconstruction.rs:1074-1078: other objects are a TypeError.
    with pytest.raises(TypeError):
        fpm.AlternatingProjection(iterations=1).run(problem, callbacks=[object()])
    with pytest.raises(fpm.UnsupportedError):
        fpm.GradientDescent(recover_illumination=True, recover_pupil=True)
    with pytest.raises(fpm.InvalidParameterError):
        fpm.GradientDescent(recover_illumination=True, illumination_step=0.0)
    # tests/reconstruction_tests.rs:2882-2887: a zero finite difference is invalid.
    with pytest.raises(fpm.InvalidParameterError):
        fpm.GradientDescent(recover_illumination=True, illumination_finite_difference=0.0)
    with pytest.raises(fpm.InvalidParameterError):
        fpm.GradientDescent(illumination_bounds=float("nan"))
    fpm.GradientDescent(recover_illumination=True, object_tv=0.1)  # device illumination recovery
    fpm.GradientDescent(object_tv=0.1, recover_pupil=True, pupil_smoothing=0.02)  # device regularisers
    with pytest.raises(ValueError):
        fpm.Mpie(loss_type="l1")


def test_error_status_mapping(fpm):
    from fpm_rs import errors

    assert isinstance(errors.from_status(1, "x"), fpm.InvalidShapeError)
    assert isinstance(errors.from_status(3, "x"), fpm.InvalidModelError)
    assert isinstance(errors.from_status(7, "x"), fpm.NumericalError)
    assert isinstance(errors.from_status(8, "x"), fpm.UnsupportedError)
    assert isinstance(errors.from_status(9, "x"), fpm.DeviceError)


def test_device_calls_fail_loudly_without_a_gpu(fpm):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(fpm.DeviceError):
        fpm.fft2(np.ones((4, 4)))


def test_model_json_round_trip(fpm, tmp_path):
    grid, ref = W.led_grid(3)
    model = fpm.compile_model(fpm.Optics(**W.OPTICS), fpm.Illumination(fpm.PlanarLEDArray(
        grid, W.PITCH, ref, fpm.ArrayPose.from_translation((0.0, 0.0, W.Z)))), (32, 32))
    path = tmp_path / "model.json"
    model.save_json(path=path)
    loaded = fpm.ImagePlaneModel.load_json(path=path)
    assert loaded.reconstruction_shape == model.reconstruction_shape
    assert np.array_equal(loaded.crop_origins, model.crop_origins)
    assert np.array_equal(loaded.subpixel_offsets, model.subpixel_offsets)
    assert np.array_equal(loaded.pupil, model.pupil)


def test_checkpoint_json_round_trip(fpm, tmp_path):
    rng = np.random.default_rng(4)
    obj = rng.standard_normal((42, 42)) + 1j * rng.standard_normal((42, 42))
    pupil = rng.standard_normal((32, 32)) + 1j * rng.standard_normal((32, 32))
    cp = fpm.ReconstructionCheckpoint(completed_iterations=3, algorithm="Mpie", object_spectrum=obj, pupil=pupil,
                                      velocity=obj * 0.5, anchor=obj * 2, momentum_counter=7,
                                      objectives=[3.0, 2.0, 1.5])
    path = tmp_path / "checkpoint_00003.json"
    cp.save(path)
    back = fpm.ReconstructionCheckpoint.load(path)
    assert back.completed_iterations == 3 and back.algorithm == "Mpie" and back.momentum_counter == 7
    assert back.format_version == 2
    for name in ("object_spectrum", "pupil", "velocity", "anchor"):
        assert np.array_equal(getattr(back, name), getattr(cp, name)), name
    assert back.objectives == [3.0, 2.0, 1.5]
    assert back.illumination_corrections is None
    # Gradient-descent illumination corrections (checkpoint.rs:44) round-trip exactly.
    corr = rng.standard_normal((9, 2)) * 0.3
    gd = fpm.ReconstructionCheckpoint(completed_iterations=1, algorithm="GradientDescent", object_spectrum=obj,
                                      pupil=pupil, objectives=[1.0], illumination_corrections=corr)
    gd.save(tmp_path / "gd.json")
    assert np.array_equal(fpm.ReconstructionCheckpoint.load(tmp_path / "gd.json").illumination_corrections, corr)
    # python/src/reconstruction.rs:839-848: a zero interval becomes one.
    assert fpm.CheckpointEvery(0, tmp_path).every == 1
    with pytest.raises(OverflowError):
        fpm.CheckpointEvery(-1, tmp_path)
    assert fpm.CheckpointEvery(2, tmp_path).path_for(2).name == "checkpoint_00002.json"


def test_direction_constructors_and_accessors_round_trip(fpm):
    # tests/geometry_tests.rs:309-333, with `values` positional as the
    # binding takes it (python/src/config.rs:490-551).
    cosines = [[0.1, -0.2], [0.0, 0.0]]
    directions = fpm.DirectionList.from_direction_cosines(np.array(cosines))
    assert np.abs(directions.direction_cosines - cosines).max() <= 1e-12
    component = fpm.DirectionList.from_component_angles_degrees(np.array([[10.0, -5.0]]))
    assert np.abs(component.component_angles_deg[0] - [10.0, -5.0]).max() <= 1e-12
    polar = fpm.DirectionList.from_polar_angles_degrees(np.array([[30.0, 120.0]]))
    assert np.abs(polar.polar_angles_deg[0] - [30.0, 120.0]).max() <= 1e-12
    normalized = fpm.DirectionList.from_vectors(np.array([[0.0, 0.0, 2.0]]))
    assert np.array_equal(normalized.unit_vectors, [[0.0, 0.0, 1.0]])
    for bad in (lambda: fpm.DirectionList.from_unit_vectors(np.array([[0.0, 0.0, 2.0]])),
                lambda: fpm.DirectionList.from_direction_cosines(np.array([[0.8, 0.8]])),
                lambda: fpm.DirectionList.from_unit_vectors(np.array([[0.0, 0.0, -1.0]]))):
        with pytest.raises(fpm.InvalidParameterError):
            bad()


def test_direction_list_angular_forms_shapes_and_arithmetic(fpm):
    # python/tests/test_configuration.py:212-218.
    polar = fpm.DirectionList.from_polar_angles_degrees(np.array([[0.0, 0.0], [30.0, 120.0]]))
    np.testing.assert_allclose(polar.polar_angles_deg, [[0.0, 0.0], [30.0, 120.0]], atol=1e-12)
    assert polar.source_count == 2 and polar.polar_angles_rad.shape == (2, 2)
    # Component angles map through sin; polar angles through (sin t cos p, sin t sin p, cos t)
    # (src/experiment/illumination.rs:133-171).
    angles = np.array([[0.01, -0.02], [0.3, 0.1]])
    component = fpm.DirectionList.from_component_angles_radians(angles)
    assert np.array_equal(component.direction_cosines, np.vectorize(math.sin)(angles))
    np.testing.assert_allclose(component.component_angles_rad, angles, atol=1e-15)
    t, p = 0.4, -2.0
    u = fpm.DirectionList.from_polar_angles_radians(np.array([[t, p]])).unit_vectors[0]
    assert u.tolist() == [math.sin(t) * math.cos(p), math.sin(t) * math.sin(p), math.cos(t)]
    # The transverse magnitude is one fused multiply-add (f64::mul_add), so
    # z = sqrt(1 - (dx^2 + dy^2)) is rounded as the reference rounds it.
    dx, dy = 0.1, 0.7
    fused = float(Fraction(dx) * Fraction(dx) + Fraction(dy * dy))
    z = fpm.DirectionList.from_direction_cosines(np.array([[dx, dy]])).unit_vectors[0, 2]
    assert z == math.sqrt(1.0 - fused)
    # Binding shape checks (python/src/config.rs:1109-1140) raise ValueError.
    for bad in (lambda: fpm.DirectionList(np.zeros((2, 2))), lambda: fpm.DirectionList.from_vectors(np.zeros((1, 2))),
                lambda: fpm.DirectionList.from_direction_cosines(np.zeros((0, 2)))):
        with pytest.raises(ValueError):
            bad()
    # Without normalisation a vector must be unit length; a zero or non-finite one is refused either way.
    for bad in (lambda: fpm.DirectionList.from_vectors(np.array([[0.0, 0.0, 2.0]]), normalize=False),
                lambda: fpm.DirectionList.from_vectors(np.zeros((1, 3))),
                lambda: fpm.DirectionList.from_polar_angles_radians(np.array([[np.inf, 0.0]]))):
        with pytest.raises(fpm.InvalidParameterError):
            bad()


def test_resolved_sources_directions_and_positions(fpm):
    # ResolvedSources getters (python/src/config.rs:913-935): LED arrays carry
    # positions and source-to-sample directions whose k-multiples are the
    # compiled k-vectors bit for bit; direction and k-vector lists carry no
    # positions (illumination.rs:240-299).
    optics = fpm.Optics(**W.OPTICS)
    pose = fpm.ArrayPose.from_translation_and_extrinsic_xyz_degrees((1e-3, -2e-3, -85e-3), (2.0, -1.0, 15.0))
    array = fpm.PlanarLEDArray((5, 7), (4e-3, 3.5e-3), (3.2, 1.7), pose)
    resolved = array.resolve(optics)
    k = 2.0 * math.pi * optics.illumination_refractive_index / optics.wavelength_vacuum_m
    assert resolved.positions_m.shape == (35, 3) and resolved.directions.shape == (35, 3)
    assert np.array_equal(k * resolved.directions[:, :2], resolved.k_vectors)
    assert np.allclose(np.linalg.norm(resolved.directions, axis=1), 1.0, atol=1e-15)
    assert np.allclose(resolved.directions, -resolved.positions_m / np.linalg.norm(resolved.positions_m, axis=1)[:, None])
    assert array.position_offsets_m.shape == (0, 3)
    directions = fpm.DirectionList.from_direction_cosines(np.array([[0.25, -0.5]]))
    from_directions = directions.resolve(optics)
    assert from_directions.positions_m is None and np.array_equal(from_directions.directions, directions.unit_vectors)
    from_k = fpm.KVectorList(from_directions.k_vectors).resolve(optics)
    assert from_k.positions_m is None
    assert np.abs(from_k.directions - directions.unit_vectors).max() <= 1e-15
    illumination = fpm.Illumination(array)
    assert illumination.geometry is array and illumination.calibration is None and illumination.acquisition is None
    assert len(fpm.MeasurementStack(np.ones((9, 4, 4)))) == 9
    # ResolvedIllumination (python/src/config.rs:968-1041, as
    # python/tests/test_configuration.py:189-205 reads it) under the unit
    # calibration and the sequential plan: frame f is source f at unit weight.
    lit = fpm.Illumination(fpm.KVectorList(np.array([[0.0, 0.0], [1.0e4, 0.0]]))).resolve(optics)
    assert lit.directions.shape == (2, 3) and lit.k_vectors.shape == (2, 2) and lit.positions_m is None
    assert lit.source_count == 2 and lit.frame_count == 2 and not lit.is_multiplexed
    assert np.array_equal(lit.source_power, [1.0, 1.0]) and np.array_equal(lit.frame_gains, [1.0, 1.0])
    assert np.array_equal(lit.dense_weights, [[1.0, 0.0], [0.0, 1.0]])
    assert [(c.source, c.intensity_weight) for f in lit.frames for c in f.contributions] == [(0, 1.0), (1, 1.0)]
    assert np.array_equal(lit.sources.k_vectors, lit.k_vectors)
    assert np.array_equal(illumination.resolve(optics).k_vectors, resolved.k_vectors)


def test_source_position_list(fpm):
    # SourcePositionList (src/experiment/illumination.rs:45-72): the LED
    # array's own positions resolve to its compiled k-vectors bit for bit,
    # and python/tests/test_configuration.py:137-144 compiles two sources.
    optics = fpm.Optics(532e-9, 0.10, 4.0, 6.5e-6)
    pose = fpm.ArrayPose.from_translation_and_extrinsic_xyz_degrees((1e-3, -2e-3, -85e-3), (2.0, -1.0, 15.0))
    array = fpm.PlanarLEDArray((5, 7), (4e-3, 3.5e-3), (3.2, 1.7), pose).resolve(optics)
    listed = fpm.SourcePositionList(array.positions_m)
    assert listed.source_count == 35 and np.array_equal(listed.positions_m, array.positions_m)
    resolved = listed.resolve(optics)
    assert np.array_equal(resolved.k_vectors, array.k_vectors) and np.array_equal(resolved.directions, array.directions)
    model = fpm.compile_model(optics, fpm.Illumination(fpm.SourcePositionList(
        np.array([[0.0, 0.0, -0.09], [0.001, 0.0, -0.09]]))), (8, 8), (16, 16))
    assert model.source_count == 2 and model.frame_count == 2
    with pytest.raises(fpm.InvalidParameterError):
        fpm.SourcePositionList(np.zeros((1, 3))).resolve(optics)
    with pytest.raises(ValueError):
        fpm.SourcePositionList(np.zeros((0, 3)))


def test_component_angle_directions_compile(fpm):
    # python/tests/test_configuration.py:97-103,168-175: two sources, two frames.
    optics = fpm.Optics(532e-9, 0.10, 4.0, 6.5e-6)
    illumination = fpm.Illumination(fpm.DirectionList.from_component_angles_radians(np.array([[0.0, 0.0],
                                                                                             [0.01, -0.01]])))
    model = fpm.compile_model(optics, illumination, (8, 8), (16, 16))
    assert model.source_count == 2 and model.frame_count == 2


def test_direction_and_kvector_resolution_use_the_illumination_index(fpm):
    # tests/geometry_tests.rs:335-358: k scales with the illumination index;
    # explicit k-vectors resolve unchanged and must propagate.
    directions = fpm.DirectionList.from_direction_cosines(values=[[0.25, -0.5]])
    air = directions.resolve(fpm.Optics(532e-9, 0.1, 4.0, 6.5e-6))
    glass_optics = fpm.Optics(532e-9, 0.1, 4.0, 6.5e-6, illumination_refractive_index=1.5)
    glass = directions.resolve(glass_optics)
    assert abs(glass.k_vectors[0, 0] - 1.5 * air.k_vectors[0, 0]) <= 1e-9
    assert np.array_equal(fpm.KVectorList(air.k_vectors).resolve(glass_optics).k_vectors, air.k_vectors)
    k_glass = 2 * np.pi * 1.5 / 532e-9
    with pytest.raises(fpm.InvalidParameterError):
        fpm.KVectorList([[k_glass * 1.01, 0.0]]).resolve(glass_optics)


LOSS_TYPES = ("amplitude_mse", "intensity_mse", "poisson_nll", "huber_amplitude")


def _loss_in_order(predicted, measured, loss_type):
    """objective.rs:27-72 restated with NumPy per value and an in-order sum."""
    p, m = predicted.ravel(), measured.ravel()
    if loss_type == "intensity_mse":
        terms = (p - m) * (p - m)
    elif loss_type == "poisson_nll":
        mean = np.maximum(p, 1e-12)
        terms = mean - np.maximum(m, 0.0) * np.array([math.log(v) for v in mean])
    else:
        r = np.sqrt(np.maximum(p, 0.0)) - np.sqrt(np.maximum(m, 0.0))
        terms = r * r if loss_type == "amplitude_mse" else np.where(np.abs(r) <= 1.0, 0.5 * r * r, np.abs(r) - 0.5)
    return np.cumsum(np.concatenate(([0.0], terms)))[-1] / p.size


def test_intensity_loss_known_values_and_errors(fpm):
    # tests/diagnostics_tests.rs:33-64, through the binding's argument order
    # intensity_loss(reference = measured, candidate = predicted).
    measured, predicted = np.array([[1.0]]), np.array([[4.0]])
    assert fpm.intensity_loss(measured, predicted, "amplitude_mse") == 1.0
    assert fpm.intensity_loss(measured, predicted, "intensity_mse") == 9.0
    assert fpm.intensity_loss(measured, predicted, "huber_amplitude") == 0.5
    assert fpm.intensity_loss(measured, predicted, "poisson_nll") == 4.0 - math.log(4.0)
    with pytest.raises(fpm.InvalidShapeError):
        fpm.intensity_loss(np.zeros((0, 2)), np.zeros((0, 2)), "amplitude_mse")
    with pytest.raises(ValueError):
        fpm.intensity_loss(np.ones((1, 1)), np.ones((1, 2)), "amplitude_mse")
    with pytest.raises(fpm.NumericalError):
        fpm.intensity_loss(np.ones((1, 1)), np.array([[np.nan]]), "amplitude_mse")
    with pytest.raises(ValueError):
        fpm.intensity_loss(np.ones((1, 1)), np.ones((1, 1)), "l1")
    # python/src/metrics.rs:256: only the value counts must agree.
    assert fpm.intensity_loss(np.ones((1, 2)), np.full((2, 1), 4.0), "intensity_mse") == 9.0


@pytest.mark.parametrize("loss_type", LOSS_TYPES)
def test_intensity_loss_sums_in_order_and_matches_the_oracle_frame_loss(fpm, loss_type):
    import helpers

    rng = np.random.default_rng(5)
    measured = rng.normal(4.0, 3.0, (64, 48))  # some negative values, which the clamps see
    predicted = rng.normal(4.0, 3.0, (64, 48))
    assert fpm.intensity_loss(measured, predicted, loss_type) == _loss_in_order(predicted, measured, loss_type)
    # One frame of the forward model against its Poisson counts: the oracle's
    # frame loss (ImagePlaneForwardModel::frame_loss, src/model/forward.rs:475-489).
    model, omodel = helpers.planar_model(fpm, 3, 32)
    spectrum = oracle.object_spectrum(W.smooth_random_object(model.reconstruction_shape, 9))
    stack = oracle.forward_stack(oracle.Problem(omodel, None), spectrum)
    counts = rng.poisson(stack * 50.0) / 50.0
    want = oracle.frame_loss(oracle.Problem(omodel, counts), spectrum, omodel["pupil"], 4, loss_type)
    got = fpm.intensity_loss(counts[4], stack[4], loss_type)
    assert abs(got - want) <= 1e-12 * abs(want)


def test_file_errors_map_to_io_and_serialization_errors(fpm, tmp_path):
    # python/src/errors.rs:17-50: Error::Io -> FpmIoError, Error::Serialization -> SerializationError.
    model = fpm.compile_model(fpm.Optics(**W.OPTICS), fpm.Illumination(fpm.PlanarLEDArray(
        (3, 3), W.PITCH, (1.0, 1.0), fpm.ArrayPose.from_translation((0.0, 0.0, W.Z)))), (32, 32))
    model.save_json(path=tmp_path / "model.json")
    loaded = fpm.ImagePlaneModel.load_json(path=tmp_path / "model.json")
    assert np.array_equal(loaded.k_vectors, model.k_vectors) and np.array_equal(loaded.pupil, model.pupil)
    (tmp_path / "bad.json").write_text("{not json")
    (tmp_path / "partial.json").write_text("{}")
    with pytest.raises(fpm.FpmIoError):
        fpm.ImagePlaneModel.load_json(path=tmp_path / "missing.json")
    with pytest.raises(fpm.SerializationError):
        fpm.ImagePlaneModel.load_json(path=tmp_path / "bad.json")
    with pytest.raises(fpm.SerializationError):
        fpm.ImagePlaneModel.load_json(path=tmp_path / "partial.json")
    with pytest.raises(fpm.FpmIoError):
        model.save_json(path=tmp_path / "no" / "such" / "model.json")
    for checkpoint in (fpm.ReconstructionCheckpoint, fpm.SpectralReconstructionCheckpoint):
        with pytest.raises(fpm.FpmIoError):
            checkpoint.load(tmp_path / "missing.json")
        with pytest.raises(fpm.SerializationError):
            checkpoint.load(tmp_path / "bad.json")
    assert issubclass(fpm.FpmIoError, fpm.FpmError) and issubclass(fpm.DatasetError, fpm.FpmError)
