"""GPU parity of narrowband spectral AP (fpm_spectral_run) against the FP64
oracle's restatement of SpectralRunner::run + SpectralAlternatingProjection.

Tolerances as for ordinary reconstruction: complex NRMSE (global-phase
aligned) <= 1e-4 per stored object after the stated passes, objectives to
1e-4 relative, the FP32 forward stack to 1e-5 relative. Resumed runs are
bit-identical to uninterrupted ones (the complex64 state is restored
exactly).
"""

from __future__ import annotations

import numpy as np
import pytest

import oracle
import spectral_cases as sc

pytestmark = pytest.mark.gpu

NRMSE = 1e-4


@pytest.fixture(scope="module")
def fpm(native_library):
    import fpm_rs

    return fpm_rs


def _case(fpm, n, *, count=3, mixed=False, local=3, shared=False, directions=sc.DIRECTIONS, gains=None,
          background=0.0, weights=(0.4, 0.8, 1.1), gain=1.7):
    channels = [fpm.SpectralChannel(channel_id=sc.CHANNEL_IDS[c], optics=fpm.Optics(
        wavelength_vacuum_m=sc.WAVELENGTHS[c], objective_na=0.12, magnification=4.0, camera_pixel_size=6.5e-6,
        defocus_distance=1e-6)) for c in range(count)]
    if mixed:
        plan = fpm.SpectralAcquisitionPlan.multiplexed(frames=[
            fpm.SpectralFrame(contributions=[(c, l, weights[c]) for c in range(count)], gain=gain, background=background)
            for l in range(local)])
    else:
        plan = fpm.SpectralAcquisitionPlan.separate(frame_counts=[local] * count)
    coupling = "shared_complex" if shared else "independent"
    model = fpm.compile_spectral_model(
        channels=channels, geometry=fpm.SpectralGeometry.shared(geometry=fpm.DirectionList.from_direction_cosines(
            values=np.asarray(directions))), acquisition=plan, image_shape=(n, n), object_coupling=coupling)
    if gains is not None:
        model = fpm.SpectralImagePlaneModel.from_compiled_channels(
            channel_ids=model.channel_ids, models=[m._replace(frame_gains=np.asarray(gains, np.float64))
                                                   for m in model.channel_models],
            acquisition=plan, object_coupling=coupling)
    omodels = sc.compile_channels(count, directions, (n, n), "smooth", frame_gains=gains)
    assert (omodels[0]["mh"], omodels[0]["mw"]) == model.reconstruction_shape
    frames = [(f.gain, f.background, f.contributions) for f in plan.frames]
    truth = sc.truth_objects(model.reconstruction_shape, model.object_count)
    data = oracle.spectral_forward(oracle.SpectralProblem(omodels, frames, shared_object=shared), sc.spectra_of(truth))
    return model, omodels, frames, data, truth


def _compare(fpm, model, omodels, frames, data, *, iterations, shared=False, masks=None, weights=None, order=None,
             initial=None):
    problem = fpm.SpectralReconstructionProblem(measurements=data, model=model, masks=masks, frame_weights=weights)
    result = fpm.SpectralAlternatingProjection(iterations=iterations).run(
        problem=problem, frame_order=order, initial_objects=initial)
    expected = oracle.spectral_run(oracle.SpectralProblem(omodels, frames, data, shared_object=shared, masks=masks,
                                                          weights=weights),
                                   iterations=iterations, order=order, initial_objects=initial)
    index = [0 if shared else c for c in range(len(model.channel_ids))]
    for c, o in enumerate(index):
        assert oracle.complex_nrmse(expected["objects"][o], result.object[c]) <= NRMSE, c
        assert oracle.complex_nrmse(expected["spectra"][o], result.object_spectrum[c]) <= NRMSE, c
    gpu = np.array([t[1] for t in result.trace])
    assert np.all(np.abs(gpu - expected["objectives"]) <= 1e-4 * np.abs(expected["objectives"]) + 1e-12)
    return result, expected


@pytest.mark.parametrize("n", [32, 64, 128, 256])
def test_separate_channels_match_oracle(fpm, n):
    model, omodels, frames, data, _ = _case(fpm, n, gains=[1.0, 0.8, 1.2])
    _compare(fpm, model, omodels, frames, data, iterations=4)


@pytest.mark.parametrize("n", [32, 128])
def test_mixed_independent_with_background_and_masks(fpm, n):
    model, omodels, frames, data, _ = _case(fpm, n, mixed=True, background=0.2)
    masks = np.ones(data.shape, np.uint8)
    masks[:, 3, 5] = 0
    masks[1, 7:9, :] = 0
    _compare(fpm, model, omodels, frames, data, iterations=5, masks=masks)


@pytest.mark.parametrize("n", [64, 256])
def test_mixed_shared_object(fpm, n):
    model, omodels, frames, data, truth = _case(fpm, n, mixed=True, shared=True, background=0.2)
    result, _ = _compare(fpm, model, omodels, frames, data, iterations=5, shared=True)
    np.testing.assert_array_equal(result.object[0], result.object[1])
    np.testing.assert_array_equal(result.object_spectrum[1], result.object_spectrum[2])
    assert not np.array_equal(result.pupils[0], result.pupils[1])


def test_shared_object_from_truth_stays_at_the_fixed_point(fpm):
    # python/tests/test_spectral.py:108-126 at an engine tile size.
    model, omodels, frames, data, truth = _case(fpm, 32, mixed=True, shared=True, background=0.2,
                                               weights=(0.4, 0.6, 0.8))
    problem = fpm.SpectralReconstructionProblem(measurements=data, model=model)
    result = fpm.SpectralAlternatingProjection(iterations=2).run(problem=problem, initial_objects=truth)
    # FP32 state: the objective is at the single-precision rounding floor.
    assert result.trace[-1][1] < 1e-9
    assert oracle.complex_nrmse(truth[0], result.object[0]) < 1e-5


def test_explicit_order_weights_and_initial_objects(fpm):
    model, omodels, frames, data, truth = _case(fpm, 32, mixed=True, local=3, background=0.1)
    weights = np.array([1.0, 0.5, 2.0])
    init = np.ascontiguousarray(truth * 0.9 + 0.05)
    _compare(fpm, model, omodels, frames, data, iterations=4, weights=weights, order=[2, 0, 1], initial=init)


def test_separate_spectral_matches_ordinary_gpu_ap(fpm):
    # The one-channel reduction (tests/spectral_tests.rs:480-556) on the device.
    model, omodels, frames, data, _ = _case(fpm, 64, gains=[1.0, 0.8, 1.2])
    problem = fpm.SpectralReconstructionProblem(measurements=data, model=model)
    result = fpm.SpectralAlternatingProjection(iterations=4).run(problem=problem)
    for c, kernel in enumerate(model.channel_models):
        ordinary = fpm.AlternatingProjection(iterations=4).run(
            fpm.ReconstructionProblem(np.ascontiguousarray(data[3 * c:3 * c + 3]), kernel))
        assert oracle.complex_nrmse(ordinary.object, result.object[c]) <= 1e-5


def test_resume_is_bitwise_and_checkpoints_are_written(fpm, tmp_path):
    model, omodels, frames, data, _ = _case(fpm, 32, mixed=True)
    problem = fpm.SpectralReconstructionProblem(measurements=data, model=model)
    straight = fpm.SpectralAlternatingProjection(iterations=6).run(problem=problem)
    staged = fpm.SpectralAlternatingProjection(iterations=6).run(problem=problem, checkpoint_directory=tmp_path,
                                                                   checkpoint_every=2)
    np.testing.assert_array_equal(straight.object_spectrum, staged.object_spectrum)
    names = sorted(p.name for p in tmp_path.iterdir())
    assert names == ["spectral_checkpoint_00002.json", "spectral_checkpoint_00004.json",
                     "spectral_checkpoint_00006.json"]
    cp = fpm.SpectralReconstructionCheckpoint.load(tmp_path / "spectral_checkpoint_00004.json")
    resumed = fpm.SpectralAlternatingProjection(iterations=6).run(problem=problem, resume=cp)
    np.testing.assert_array_equal(straight.object_spectrum, resumed.object_spectrum)
    np.testing.assert_array_equal([t[1] for t in straight.trace], [t[1] for t in resumed.trace])
    with pytest.raises(fpm.FpmError):
        fpm.SpectralAlternatingProjection(iterations=6, object_step=0.5).run(problem=problem, resume=cp)


@pytest.mark.parametrize("n", [32, 128])
def test_forward_intensities_match_oracle(fpm, n):
    model, omodels, frames, data, truth = _case(fpm, n, mixed=True, background=0.2, gains=[1.3, 0.7, 1.0])
    gpu = model.forward_intensities(object_spectra=sc.spectra_of(truth))
    assert np.abs(gpu - data).max() <= 1e-5 * np.abs(data).max()


def test_bounded_rgb_multiplexed_recovery(fpm):
    # tests/spectral_tests.rs:819-898 at a 32-pixel tile.
    directions = [(dx, dy) for dy in (-0.12, 0.0, 0.12) for dx in (-0.12, 0.0, 0.12)]
    channels = [fpm.SpectralChannel(channel_id=sc.CHANNEL_IDS[c], optics=fpm.Optics(
        wavelength_vacuum_m=sc.WAVELENGTHS[c], objective_na=0.12, magnification=4.0, camera_pixel_size=6.5e-6))
        for c in range(3)]
    plan = fpm.SpectralAcquisitionPlan.multiplexed(frames=[
        fpm.SpectralFrame(contributions=[(c, l, 1.0 if c == dominant else 0.1) for c in range(3)])
        for l in range(9) for dominant in range(3)])
    model = fpm.compile_spectral_model(
        channels=channels, geometry=fpm.SpectralGeometry.shared(
            geometry=fpm.DirectionList.from_direction_cosines(values=np.asarray(directions))),
        acquisition=plan, image_shape=(32, 32))
    mh, mw = model.reconstruction_shape
    rows, cols = np.indices((mh, mw))
    x, y = 2 * np.pi * cols / mw, 2 * np.pi * rows / mh
    truth = np.stack([(0.65 + c * 0.12 + 0.08 * np.cos(x + c)) * np.exp(1j * 0.08 * np.sin(2 * y + c))
                      for c in range(3)])
    spectra = np.ascontiguousarray(sc.spectra_of(truth))
    data = model.forward_intensities(object_spectra=spectra)
    result = fpm.SpectralAlternatingProjection(iterations=150).run(
        problem=fpm.SpectralReconstructionProblem(measurements=data, model=model))
    assert result.trace[-1][1] < result.trace[0][1] * 0.01
    for c in range(3):
        assert oracle.complex_nrmse(truth[c], result.object[c]) < 0.03


def test_batched_requests_equal_single_runs(fpm):
    # Mixed tile sizes and couplings in one call: one launch per size.
    cases = [_case(fpm, 32, mixed=True), _case(fpm, 64, gains=[1.0, 0.8, 1.2]),
             _case(fpm, 32, mixed=True, shared=True, background=0.2), _case(fpm, 128, mixed=True)]
    problems = [fpm.SpectralReconstructionProblem(measurements=c[3], model=c[0]) for c in cases]
    solver = fpm.SpectralAlternatingProjection(iterations=3)
    batch = solver.run_many(problems=problems)
    stats = fpm.last_run_stats()
    assert stats["engine_launches"] == 3
    assert [b[:2] for b in stats["buckets"]] == [(128, 1), (64, 1), (32, 2)]
    for problem, got in zip(problems, batch):
        alone = solver.run(problem=problem)
        np.testing.assert_array_equal(alone.object_spectrum, got.object_spectrum)
        np.testing.assert_array_equal([t[1] for t in alone.trace], [t[1] for t in got.trace])
