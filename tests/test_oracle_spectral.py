"""The FP64 oracle's narrowband spectral AP, pinned by the reference's own
spectral properties (tests/spectral_tests.rs:480-898,
python/tests/test_spectral.py:66-147): reduction to ordinary AP, mixed
forward composition, mask invariance, channel-permutation invariance, the
shared-object fixed point and bounded RGB recovery."""

import numpy as np
import pytest

import oracle
import spectral_cases as sc


def _forward(channels, frames, objects, shared=False):
    problem = oracle.SpectralProblem(channels, frames, shared_object=shared)
    return oracle.spectral_forward(problem, sc.spectra_of(objects))


def test_single_channel_matches_ordinary_ap_with_gains():
    # tests/spectral_tests.rs:480-517 (frame gains stand in for source powers)
    ch = sc.compile_channels(count=1, frame_gains=[1.0, 0.8, 1.2])
    frames = sc.separate_frames([3])
    truth = sc.truth_objects((ch[0]["mh"], ch[0]["mw"]), 1)
    data = _forward(ch, frames, truth)
    spectral = oracle.spectral_run(oracle.SpectralProblem(ch, frames, data), iterations=4)
    ordinary = oracle.run(oracle.Problem(ch[0], data, gains=ch[0]["frame_gains"]), "ap", iterations=4)
    np.testing.assert_array_equal(spectral["spectra"][0], ordinary["object_spectrum"])
    np.testing.assert_array_equal(spectral["objectives"], ordinary["objectives"])


def test_separate_channels_match_per_channel_ap():
    # tests/spectral_tests.rs:519-556
    ch = sc.compile_channels(count=3)
    frames = sc.separate_frames([3, 3, 3])
    truth = sc.truth_objects((ch[0]["mh"], ch[0]["mw"]), 3)
    data = _forward(ch, frames, truth)
    result = oracle.spectral_run(oracle.SpectralProblem(ch, frames, data), iterations=4)
    for c in range(3):
        ordinary = oracle.run(oracle.Problem(ch[c], np.ascontiguousarray(data[3 * c:3 * c + 3])), "ap", iterations=4)
        np.testing.assert_array_equal(result["spectra"][c], ordinary["object_spectrum"])


def test_union_grid_and_wavelength_scaled_kvectors():
    # tests/spectral_tests.rs:429-478
    ch = sc.compile_channels(count=3, policy="smooth")
    for c in range(3):
        k = sc.kvectors(sc.WAVELENGTHS[c], sc.DIRECTIONS)
        alone = oracle.compile_model(sc.optics(sc.WAVELENGTHS[c]), k[:, 0], k[:, 1], (8, 12), "minimum")
        assert ch[c]["mh"] >= alone["mh"]
        np.testing.assert_array_equal(ch[c]["pupil"], alone["pupil"])
    assert not np.array_equal(ch[0]["support"], ch[2]["support"])
    assert abs(ch[0]["kx"][1] / ch[2]["kx"][1] - 630.0 / 450.0) < 1e-14
    with pytest.raises(oracle.OracleError):
        k = np.concatenate([sc.kvectors(w, sc.DIRECTIONS) for w in sc.WAVELENGTHS])
        oracle.compile_model(sc.optics(450e-9), k[:, 0], k[:, 1], (8, 12), (8, 12))


def test_mixed_forward_matches_manual_channel_sum():
    # tests/spectral_tests.rs:558-586
    ch = sc.compile_channels(count=3, frame_gains=[1.3, 0.7, 1.0])
    frames = sc.mixed_frames()
    truth = sc.truth_objects((ch[0]["mh"], ch[0]["mw"]), 3)
    got = _forward(ch, frames, truth)
    spectra = sc.spectra_of(truth)
    for e, (gain, background, contributions) in enumerate(frames):
        total = np.zeros((8, 12))
        for c, l, w in contributions:
            local = oracle.forward_stack(oracle.Problem(ch[c], None, gains=ch[c]["frame_gains"]), spectra[c])[l]
            total = total + w * local
        np.testing.assert_array_equal(got[e], gain * total + background)


def test_shared_object_fixed_point_and_descent():
    # python/tests/test_spectral.py:108-126 and tests/spectral_tests.rs:588-607
    ch = sc.compile_channels(count=3)
    frames = [(1.7, 0.2, [(c, l, 0.4 + 0.2 * c) for c in range(3)]) for l in range(3)]
    truth = sc.truth_objects((ch[0]["mh"], ch[0]["mw"]), 1)
    data = _forward(ch, frames, truth, shared=True)
    problem = oracle.SpectralProblem(ch, frames, data, shared_object=True)
    exact = oracle.spectral_run(problem, iterations=2, initial_objects=truth)
    assert exact["objectives"][-1] < 1e-16
    run = oracle.spectral_run(problem, iterations=8)
    assert run["objectives"][-1] < run["objectives"][0]


def test_masked_pixels_do_not_affect_any_object():
    # tests/spectral_tests.rs:726-753
    ch = sc.compile_channels(count=3)
    frames = sc.mixed_frames()
    truth = sc.truth_objects((ch[0]["mh"], ch[0]["mw"]), 3)
    data = _forward(ch, frames, truth)
    masks = np.ones(data.shape, np.uint8)
    masks[:, 3, 5] = 0
    changed = data.copy()
    changed[:, 3, 5] = 1e6
    a = oracle.spectral_run(oracle.SpectralProblem(ch, frames, data, masks=masks), iterations=3)
    b = oracle.spectral_run(oracle.SpectralProblem(ch, frames, changed, masks=masks), iterations=3)
    np.testing.assert_array_equal(a["spectra"], b["spectra"])
    assert a["objectives"][-1] == b["objectives"][-1]


def test_permuting_channels_preserves_predictions_and_recovery():
    # tests/spectral_tests.rs:755-817
    ch = sc.compile_channels(count=3)
    frames = sc.mixed_frames()
    truth = sc.truth_objects((ch[0]["mh"], ch[0]["mw"]), 3)
    data = _forward(ch, frames, truth)
    order = [2, 0, 1]
    ch2 = [ch[i] for i in order]
    frames2 = [(g, b, sorted((order.index(c), l, w) for c, l, w in contributions))
               for g, b, contributions in frames]
    data2 = _forward(ch2, frames2, truth[order])
    np.testing.assert_allclose(data2, data, rtol=0, atol=1e-14)
    a = oracle.spectral_run(oracle.SpectralProblem(ch, frames, data), iterations=3)
    b = oracle.spectral_run(oracle.SpectralProblem(ch2, frames2, data), iterations=3)
    for new, old in enumerate(order):
        assert np.max(np.abs(a["objects"][old] - b["objects"][new])) < 1e-13


def test_bounded_rgb_multiplexed_recovery():
    # tests/spectral_tests.rs:819-898
    directions = [(dx, dy) for dy in (-0.12, 0.0, 0.12) for dx in (-0.12, 0.0, 0.12)]
    ch = sc.compile_channels(count=3, directions=directions, defocus=None)
    frames = [(1.0, 0.0, [(c, l, 1.0 if c == dominant else 0.1) for c in range(3)])
              for l in range(9) for dominant in range(3)]
    mh, mw = ch[0]["mh"], ch[0]["mw"]
    rows, cols = np.indices((mh, mw))
    x = 2 * np.pi * cols / mw
    y = 2 * np.pi * rows / mh
    truth = np.stack([(0.65 + c * 0.12 + 0.08 * np.cos(x + c)) * np.exp(1j * 0.08 * np.sin(2 * y + c))
                      for c in range(3)])
    data = _forward(ch, frames, truth)
    result = oracle.spectral_run(oracle.SpectralProblem(ch, frames, data), iterations=150)
    assert result["objectives"][-1] < result["objectives"][0] * 0.01
    for c in range(3):
        assert oracle.complex_nrmse(truth[c], result["objects"][c]) < 0.03
