"""Host-side spectral API: plan canonicalisation and validation
(tests/spectral_tests.rs:609-724, python/tests/test_spectral.py:129-192),
the common union grid against the oracle's compilation, and the checkpoint
file format. No GPU is used."""

import numpy as np
import pytest

import spectral_cases as sc


@pytest.fixture(scope="module")
def fpm(native_library):
    import fpm_rs

    return fpm_rs


def _channels(fpm, count=3, wavelengths=sc.WAVELENGTHS, magnification=4.0):
    return [fpm.SpectralChannel(channel_id=sc.CHANNEL_IDS[c], optics=fpm.Optics(
        wavelength_vacuum_m=wavelengths[c], objective_na=0.12, magnification=magnification,
        camera_pixel_size=6.5e-6, defocus_distance=1e-6)) for c in range(count)]


def _geometry(fpm):
    return fpm.SpectralGeometry.shared(geometry=fpm.DirectionList.from_direction_cosines(values=np.asarray(sc.DIRECTIONS)))


def test_plan_canonicalisation_and_rejections(fpm):
    plan = fpm.SpectralAcquisitionPlan.multiplexed(
        frames=[fpm.SpectralFrame(contributions=[(0, 0, 0.2), (0, 0, 0.3), (4, 9, 0.0)])])
    assert plan.frames[0].contributions == [(0, 0, 0.5)]
    plan = fpm.SpectralAcquisitionPlan.multiplexed(
        frames=[fpm.SpectralFrame(contributions=[(2, 1, 0.5), (0, 3, 1.0), (1, 0, 0.25)])])
    assert plan.frames[0].contributions == [(0, 3, 1.0), (1, 0, 0.25), (2, 1, 0.5)]
    for weight in (-1.0, float("nan"), float("inf")):
        with pytest.raises(fpm.FpmError):
            fpm.SpectralAcquisitionPlan.multiplexed(frames=[fpm.SpectralFrame(contributions=[(0, 0, weight)])])
    with pytest.raises(fpm.FpmError):
        fpm.SpectralAcquisitionPlan.multiplexed(frames=[fpm.SpectralFrame(contributions=[(0, 0, 0.0)])])
    with pytest.raises(fpm.FpmError):
        fpm.SpectralAcquisitionPlan.multiplexed(frames=[fpm.SpectralFrame(contributions=[(0, 0, 1.0)], gain=0.0)])
    with pytest.raises(fpm.FpmError):
        fpm.SpectralAcquisitionPlan.separate(frame_counts=[2, 0])
    assert fpm.SpectralAcquisitionPlan.separate(frame_counts=[2, 1]).frame_count == 3


def test_union_grid_matches_oracle_compilation(fpm):
    model = fpm.compile_spectral_model(channels=_channels(fpm), geometry=_geometry(fpm),
                                       acquisition=fpm.SpectralAcquisitionPlan.separate(frame_counts=[3, 3, 3]),
                                       image_shape=(8, 12))
    ref = sc.compile_channels(3)
    assert model.reconstruction_shape == (ref[0]["mh"], ref[0]["mw"])
    for c, m in enumerate(model.channel_models):
        np.testing.assert_array_equal(m.crop_origins[:, 0], ref[c]["start_row"])
        np.testing.assert_array_equal(m.crop_origins[:, 1], ref[c]["start_col"])
        np.testing.assert_array_equal(m.subpixel_offsets[:, 0], ref[c]["off_row"])
        np.testing.assert_array_equal(m.subpixel_offsets[:, 1], ref[c]["off_col"])
        np.testing.assert_array_equal(m.pupil, ref[c]["pupil"])
    assert model.channel_ids == ["blue", "green", "red"]
    assert model.wavelengths_vacuum_m == list(sc.WAVELENGTHS)
    blue, red = model.channel_models[0], model.channel_models[2]
    assert abs(blue.k_vectors[1, 0] / red.k_vectors[1, 0] - 630.0 / 450.0) < 1e-14
    with pytest.raises(fpm.FpmError):
        fpm.compile_spectral_model(channels=_channels(fpm), geometry=_geometry(fpm),
                                   acquisition=fpm.SpectralAcquisitionPlan.separate(frame_counts=[3, 3, 3]),
                                   image_shape=(8, 12), reconstruction_shape=(8, 12))


def test_invalid_channel_sets_are_rejected(fpm):
    plan = fpm.SpectralAcquisitionPlan.separate(frame_counts=[3, 3, 3])

    def build(channels, geometry=None):
        return fpm.compile_spectral_model(channels=channels, geometry=geometry or _geometry(fpm), acquisition=plan,
                                          image_shape=(8, 12))

    chans = _channels(fpm)
    chans[1]._channel_id = chans[0].channel_id
    with pytest.raises(fpm.FpmError):
        build(chans)
    with pytest.raises(fpm.FpmError):
        build(_channels(fpm, wavelengths=(450e-9, 450e-9, 630e-9)))
    odd = _channels(fpm)
    odd[1] = _channels(fpm, magnification=5.0)[1]
    with pytest.raises(fpm.FpmError, match="sampling"):
        build(odd)
    with pytest.raises(fpm.FpmError, match="cannot be shared"):
        build(_channels(fpm), fpm.SpectralGeometry.shared(geometry=fpm.KVectorList(np.zeros((3, 2)))))
    with pytest.raises(fpm.FpmError, match="out of range"):
        fpm.compile_spectral_model(channels=_channels(fpm), geometry=_geometry(fpm), image_shape=(8, 12),
                                   acquisition=fpm.SpectralAcquisitionPlan.multiplexed(
                                       frames=[fpm.SpectralFrame(contributions=[(0, 9, 1.0)])]))
    with pytest.raises(fpm.FpmError, match="participate"):
        fpm.compile_spectral_model(channels=_channels(fpm), geometry=_geometry(fpm), image_shape=(8, 12),
                                   acquisition=fpm.SpectralAcquisitionPlan.separate(frame_counts=[3, 3, 2]))


def test_problem_validation_and_run_arguments(fpm):
    plan = fpm.SpectralAcquisitionPlan.multiplexed(frames=[
        fpm.SpectralFrame(contributions=[(c, l, 0.4 + 0.2 * c) for c in range(3)], gain=1.7, background=0.2)
        for l in range(3)])
    model = fpm.compile_spectral_model(channels=_channels(fpm), geometry=_geometry(fpm), acquisition=plan,
                                       image_shape=(8, 12))
    data = np.ones((3, 8, 12))
    with pytest.raises(fpm.FpmError, match="positive-weight"):
        fpm.SpectralReconstructionProblem(measurements=data, model=model, frame_weights=[1.0, 0.0, 1.0])
    masks = np.ones((3, 8, 12), np.uint8)
    masks[1] = 0
    with pytest.raises(fpm.FpmError, match="no unmasked"):
        fpm.SpectralReconstructionProblem(measurements=data, model=model, masks=masks)
    with pytest.raises(fpm.FpmError):
        fpm.SpectralReconstructionProblem(measurements=np.ones((2, 8, 12)), model=model)
    problem = fpm.SpectralReconstructionProblem(measurements=data, model=model)
    solver = fpm.SpectralAlternatingProjection(iterations=1)
    objects = np.ones((3, *model.reconstruction_shape), np.complex128)
    with pytest.raises(fpm.FpmError, match="contiguous"):
        solver.run(problem=problem, initial_objects=objects[:, :, ::-1])
    with pytest.raises(fpm.FpmError, match="permutation"):
        solver.run(problem=problem, frame_order=[0, 0, 2])
    with pytest.raises(ValueError, match="mutually exclusive"):
        solver.run(problem=problem, frame_order=[0, 1, 2], seed=1)
    with pytest.raises(fpm.UnsupportedError):
        solver.run(problem=problem, seed=1)
    for bad in (dict(iterations=0), dict(object_step=0.0), dict(epsilon=float("nan")), dict(batch_size=0)):
        with pytest.raises(fpm.FpmError):
            fpm.SpectralAlternatingProjection(**bad).run(problem=problem)
    with pytest.raises(fpm.FpmError, match="contiguous"):
        model.forward_intensities(object_spectra=objects[:, :, ::-1])


def test_mixing_diagnostics(fpm):
    plan = fpm.SpectralAcquisitionPlan.multiplexed(frames=[
        fpm.SpectralFrame(contributions=[(0, l, 3.0), (1, l, 0.0 + 1e-300)]) for l in range(3)] + [
        fpm.SpectralFrame(contributions=[(1, l, 1.0)]) for l in range(3)])
    model = fpm.compile_spectral_model(channels=_channels(fpm, count=2), geometry=_geometry(fpm), acquisition=plan,
                                       image_shape=(8, 12))
    d = model.mixing_diagnostics()
    assert d.matrix.shape == (6, 2)
    assert d.rank == 2
    assert d.channel_ids == ["blue", "green"]
    assert abs(d.condition_number - 3.0) < 1e-12
    assert model.mixing_diagnostics(relative_tolerance=0.5).rank == 1


def test_checkpoint_round_trip(fpm, tmp_path):
    cp = fpm.SpectralReconstructionCheckpoint(
        completed_iterations=2, elapsed_seconds=0.5, spectra=np.arange(12).reshape(1, 3, 4) * (1 + 2j),
        trace=[(1, 0.5, 0.1), (2, 0.25, 0.2)], configuration=dict(object_step=1.0, batch_size=1, epsilon=1e-10,
                                                                   loss_type="amplitude_mse"),
        schedule=[1, 0], model_fingerprint="m", measurement_fingerprint="d")
    cp.save(tmp_path / "spectral_checkpoint_00002.json")
    back = fpm.SpectralReconstructionCheckpoint.load(tmp_path / "spectral_checkpoint_00002.json")
    np.testing.assert_array_equal(back.spectra, cp.spectra)
    assert back.trace == cp.trace and back.schedule == [1, 0] and back.configuration == cp.configuration
