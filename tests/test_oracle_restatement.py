"""A second restatement of the projection algorithms, in NumPy and independent
of the C oracle, written from the reference's Rust:

- state initialisation: src/reconstruction/state.rs:280-349;
- projection_update: src/algorithms/common.rs:57-306 (one source per frame);
- mPIE momentum: common.rs:308-387 and src/algorithms/mpie.rs:152-164;
- the crop and its exact adjoint: src/model/crop.rs:79-313;
- the point loss: src/algorithms/objective.rs:47-72;
- the per-pass objective: src/algorithms/metrics.rs:24-35;
- the result object: src/reconstruction/result.rs:397-413.

Each run's per-pass objectives and final object must agree with the oracle's
to rounding. The two share no code: NumPy's FFT here, the oracle's own FFT
there. So the oracle's reading of the reference, which the GPU parity tests
rest on, is checked by a second reading over whole trajectories.
"""

from __future__ import annotations

import math

import numpy as np
import pytest

import helpers
import oracle
import workloads as W

EPS = 1e-10


def _round_half_away(x: float) -> float:
    return math.copysign(math.floor(abs(x) + 0.5), x)


def _axis(start: int, length: int, offset: float):
    """interpolation_axis (crop.rs:258-313): lower start, upper start and weights."""
    nearest = _round_half_away(offset)
    if abs(offset - nearest) <= 1e-12:
        whole, fraction = nearest, 0.0
    else:
        whole = math.floor(offset)
        fraction = offset - whole
    lower = start + int(whole)
    return lower, lower + (1 if fraction > 0.0 else 0), 1.0 - fraction, fraction


def _stencil(model, source, offset=None):
    h, w = model["h"], model["w"]
    sr, sc = int(model["start_row"][source]), int(model["start_col"][source])
    orow, ocol = ((float(model["off_row"][source]), float(model["off_col"][source])) if offset is None
                  else offset)
    if abs(orow) <= 1e-12 and abs(ocol) <= 1e-12:
        return [(sr, sc, 1.0)], h, w
    lr, ur, lwr, uwr = _axis(sr, h, orow)
    lc, uc, lwc, uwc = _axis(sc, w, ocol)
    return [(lr, lc, lwr * lwc), (lr, uc, lwr * uwc), (ur, lc, uwr * lwc), (ur, uc, uwr * uwc)], h, w


def _offset_inside(model, source, offset):
    """validate_subpixel_inside (crop.rs:104-113, :286-305) on both axes."""
    for start, length, bound, value in ((int(model["start_row"][source]), model["h"], model["mh"], offset[0]),
                                        (int(model["start_col"][source]), model["w"], model["mw"], offset[1])):
        lower, upper, _, fraction = _axis(start, length, value)
        if lower < 0 or lower + length > bound or (fraction > 0.0 and lower + length >= bound):
            return False
    return True


def _extract(spectrum, model, source, offset=None):
    taps, h, w = _stencil(model, source, offset)
    out = np.zeros((h, w), np.complex128)
    for r, c, weight in taps:
        out = out + spectrum[r:r + h, c:c + w] * weight
    return out


def _insert_adjoint(spectrum, model, source, update, scale, offset=None):
    taps, h, w = _stencil(model, source, offset)
    value = scale * update
    for r, c, weight in taps:
        spectrum[r:r + h, c:c + w] += value * weight


def _point_loss(predicted, measured, loss):
    if loss == "intensity_mse":
        return (predicted - measured) ** 2
    if loss == "poisson_nll":
        mean = np.maximum(predicted, 1e-12)
        return mean - np.maximum(measured, 0.0) * np.log(mean)
    r = np.sqrt(np.maximum(predicted, 0.0)) - np.sqrt(np.maximum(measured, 0.0))
    if loss == "amplitude_mse":
        return r * r
    return np.where(np.abs(r) <= 1.0, 0.5 * r * r, np.abs(r) - 0.5)


def _fft_forward(x):
    return np.fft.fft2(x) / x.size


def _fft_inverse(x):
    return np.fft.ifft2(x) * x.size


def _initial_spectrum(model, data, gains, weights, masks, background):
    h, w, mh, mw = model["h"], model["w"], model["mh"], model["mw"]
    average = np.zeros((h, w))
    weight = np.zeros((h, w))
    total_amplitude = total_weight = 0.0
    for f in range(data.shape[0]):
        if weights[f] == 0.0:
            continue
        valid = np.ones((h, w), bool) if masks is None else masks[f] != 0
        amplitude = np.sqrt(np.maximum((data[f] - background[f]) / gains[f], 0.0))
        average[valid] += weights[f] * amplitude[valid]
        weight[valid] += weights[f]
        total_amplitude += float(np.sum(weights[f] * amplitude[valid]))
        total_weight += weights[f] * int(valid.sum())
    average = np.where(weight > 0.0, average / np.where(weight > 0.0, weight, 1.0), total_amplitude / total_weight)
    rows = (np.arange(mh) * h) // mh
    cols = (np.arange(mw) * w) // mw
    obj = average[rows[:, None], cols[None, :]].astype(np.complex128)
    return np.fft.fftshift(_fft_forward(obj))


def restated_run(model, data, algorithm, iterations, *, loss="amplitude_mse", weights=None, masks=None,
                 gains=None, background=None, recover_gains=False, recover_background=False, order=None,
                 initial_spectrum=None, progress_threshold=0.01, reduction_factor=0.5, minimum_object_step=0.001,
                 recover_pupil=False, pupil_step=0.1, canonicalize=None):
    """AP / adaptive AP / FPIE / mPIE / EPRY with the reference defaults,
    batch 1; EPRY optionally recovers frame gains and backgrounds
    (update_gain / update_background, common.rs:389-489) and the pupil
    (common.rs:272-302), the runner then canonicalising object and pupil after
    initialisation and after every pass through `canonicalize`."""
    frames = data.shape[0]
    weights = np.ones(frames) if weights is None else np.asarray(weights, np.float64)
    gains = np.ones(frames) if gains is None else np.array(gains, np.float64)
    bg = np.zeros((frames, model["h"], model["w"])) if background is None else np.array(background, np.float64)
    step, denominator, alpha, momentum = {
        "ap": (1.0, "local", 0.0, False),
        "fpie": (0.8, "rpie", 0.1, False),
        "mpie": (0.2, "rpie", 0.05, True),
        "epry": (0.8, "global", 0.0, False),
        "adaptive_ap": (1.0, "local", 0.0, False),
    }[algorithm]
    spectrum = (_initial_spectrum(model, data, gains, weights, masks, bg) if initial_spectrum is None
                else np.array(initial_spectrum, np.complex128))
    pupil = np.array(model["pupil"], np.complex128)
    support = np.asarray(model["support"]) != 0
    if recover_pupil and canonicalize is not None:
        spectrum, pupil = canonicalize(spectrum, pupil)
    velocity = np.zeros_like(spectrum)
    anchor = spectrum.copy()
    counter = 0
    objectives = []
    steps = []
    for i in range(iterations):
        if algorithm == "adaptive_ap" and i >= 2:
            # AdaptiveAlternatingProjection::begin_iteration (adaptive_alternating_projection.rs:245-307).
            progress = (objectives[-2] - objectives[-1]) / max(objectives[-2], EPS)
            if progress <= progress_threshold:
                step = max(step * reduction_factor, minimum_object_step)
        steps.append(step)
        objective_sum = weight_sum = 0.0
        for f in (range(frames) if order is None else order):
            fw = weights[f]
            if fw == 0.0:
                continue
            patch = _extract(spectrum, model, f)
            field = _fft_inverse(np.fft.ifftshift(patch * pupil))
            intrinsic = np.abs(field) ** 2
            valid = np.ones(intrinsic.shape, bool) if masks is None else masks[f] != 0
            if recover_gains:
                numerator = float(np.sum((intrinsic * np.maximum(data[f] - bg[f], 0.0))[valid]))
                den_sum = float(np.sum((intrinsic * intrinsic)[valid]))
                if den_sum > EPS:
                    estimate = min(max(numerator / den_sum, 1e-6), 1e6)
                    gains[f] = min(max(0.8 * gains[f] + 0.2 * estimate, 1e-6), 1e6)
            if recover_background:
                residual = float(np.sum((data[f] - gains[f] * intrinsic - bg[f])[valid]))
                bg[f] = np.clip(bg[f] + 0.2 * residual / int(valid.sum()), 0.0, 1e12)
            predicted = gains[f] * intrinsic + bg[f]
            frame_loss = float(np.sum(_point_loss(predicted, data[f], loss)[valid]))
            objective_sum += fw * (frame_loss / int(valid.sum()))
            weight_sum += fw
            target = np.maximum((data[f] - bg[f]) / gains[f], 0.0)
            bright = intrinsic > EPS
            ratio = np.sqrt(target / np.where(bright, intrinsic, 1.0))
            difference = np.where(bright, field * ratio, np.sqrt(target) + 0j)
            difference = np.where(valid, difference, field)
            projected = np.fft.fftshift(_fft_forward(difference))
            delta = projected - patch * pupil
            power = np.abs(pupil) ** 2
            maximum = max(float(power.max()), EPS)
            if denominator == "local":
                den = power + EPS
            elif denominator == "global":
                den = maximum + EPS
            else:
                den = (1.0 - alpha) * power + alpha * maximum + EPS
            _insert_adjoint(spectrum, model, f, np.conj(pupil) * delta / den, fw * step)
            if recover_pupil:
                object_power = max(float((np.abs(patch) ** 2).max()), EPS)
                pupil = pupil + fw * pupil_step * (np.conj(patch) * delta / (object_power + EPS))
                pupil = np.where(support, pupil, 0.0)
            if momentum:
                counter += 1
                if counter == 30:
                    velocity = 0.9 * velocity + (spectrum - anchor)
                    spectrum = spectrum + 0.9 * velocity
                    anchor = spectrum.copy()
                    counter = 0
        if recover_pupil and canonicalize is not None:
            spectrum, pupil = canonicalize(spectrum, pupil)
        objectives.append(objective_sum / weight_sum)
    return dict(objectives=np.array(objectives), object_spectrum=spectrum,
                object=_fft_inverse(np.fft.ifftshift(spectrum)), frame_gains=gains, background=bg,
                object_steps=np.array(steps), pupil=pupil)


def _descent_factor(predicted, measured, loss):
    """descent_factor (src/algorithms/gradient_descent.rs:1167-1178)."""
    if loss == "amplitude_mse":
        return 1.0 - np.sqrt(np.maximum(measured, 0.0)) / np.sqrt(np.maximum(predicted, EPS))
    if loss == "intensity_mse":
        return 2.0 * (predicted - measured)
    if loss == "poisson_nll":
        return 1.0 - np.maximum(measured, 0.0) / np.maximum(predicted, EPS)
    amplitude = np.sqrt(np.maximum(predicted, EPS))
    return np.clip(amplitude - np.sqrt(np.maximum(measured, 0.0)), -1.0, 1.0) / (2.0 * amplitude)


def _tv_gradient(values, epsilon):
    """apply_complex_tv_step's gradient (src/algorithms/regularization.rs:5-45):
    forward differences, each pixel's pair normalised by
    sqrt(|dx|^2 + |dy|^2 + eps^2), scattered back with opposite signs."""
    dh = np.zeros_like(values)
    dv = np.zeros_like(values)
    dh[:, :-1] = values[:, 1:] - values[:, :-1]
    dv[:-1, :] = values[1:, :] - values[:-1, :]
    norm = np.sqrt(np.abs(dh) ** 2 + np.abs(dv) ** 2 + epsilon * epsilon)
    nh, nv = dh / norm, dv / norm
    gradient = -nh - nv
    gradient[:, 1:] += nh[:, :-1]
    gradient[1:, :] += nv[:-1, :]
    return gradient


def _smoothing_gradient(values):
    """apply_quadratic_smoothing_step's gradient (regularization.rs:47-76)."""
    dh = np.zeros_like(values)
    dv = np.zeros_like(values)
    dh[:, :-1] = values[:, 1:] - values[:, :-1]
    dv[:-1, :] = values[1:, :] - values[:-1, :]
    gradient = -2.0 * dh - 2.0 * dv
    gradient[:, 1:] += 2.0 * dh[:, :-1]
    gradient[1:, :] += 2.0 * dv[:-1, :]
    return gradient


def restated_gd(model, data, iterations, batch_size, *, loss="amplitude_mse", weights=None, masks=None,
                gains=None, background=None, object_step=0.5, order=None, recover_pupil=False, pupil_step=0.05,
                truncation_threshold=None, canonicalize=None, object_tv=0.0, object_tv_epsilon=1e-6,
                pupil_smoothing=0.0, recover_illumination=False, illumination_step=0.1,
                illumination_finite_difference=0.05, illumination_bounds=1.0):
    """GradientDescent::step (gradient_descent.rs:405-671) without truncation,
    pupil or illumination recovery, or regularisers: per batch, the frames'
    Wirtinger gradients accumulate, each frame scaled by its weight times
    N / (valid pixels), then the object takes one step of object_step over
    the batch's active frame count. The loss compares |psi|^2 with
    (I - background) / gain. Optionally the pupil descends too (its gradient
    over max |patch|^2, stepped after the batch, then the support applied),
    and Poisson truncation (compute_truncation_statistics, :701-791) drops
    pixels with |target - prediction| > scale * sqrt(prediction) from the
    gradient, the scale taken from the pre-batch state. With pupil recovery
    the runner canonicalises object and pupil after initialisation and after
    every pass (src/reconstruction/runner.rs:122,220); `canonicalize` is that
    gauge (src/algorithms/gauge.rs), which this file does not restate."""
    frames = data.shape[0]
    weights = np.ones(frames) if weights is None else np.asarray(weights, np.float64)
    gains = np.ones(frames) if gains is None else np.asarray(gains, np.float64)
    bg = np.zeros((frames, model["h"], model["w"])) if background is None else background
    spectrum = _initial_spectrum(model, data, gains, weights, masks, bg)
    pupil = np.array(model["pupil"], np.complex128)
    support = np.asarray(model["support"]) != 0
    n = model["h"] * model["w"]
    objectives = []
    rejected = 0
    corrections = np.zeros((frames, 2))
    if recover_pupil and canonicalize is not None:
        spectrum, pupil = canonicalize(spectrum, pupil)

    def offset_of(f, extra=(0.0, 0.0)):
        """effective_source_offset (state.rs:245-267): compiled offset plus correction."""
        return (float(model["off_row"][f]) + corrections[f, 0] + extra[0],
                float(model["off_col"][f]) + corrections[f, 1] + extra[1])

    def intensity_at(f, offset):
        return np.abs(_fft_inverse(np.fft.ifftshift(_extract(spectrum, model, f, offset) * pupil))) ** 2

    def frame_terms(f):
        patch = _extract(spectrum, model, f, offset_of(f))
        field = _fft_inverse(np.fft.ifftshift(patch * pupil))
        valid = np.ones(field.shape, bool) if masks is None else masks[f] != 0
        target = np.maximum((data[f] - bg[f]) / gains[f], 0.0)
        return patch, field, np.maximum(np.abs(field) ** 2, 0.0), valid, target
    for _ in range(iterations):
        objective_sum = weight_sum = 0.0
        sequence = list(range(frames)) if order is None else list(order)
        for first in range(0, frames, batch_size):
            batch = [f for f in sequence[first:first + batch_size]]
            scale = None
            if truncation_threshold is not None:
                residual = weight_total = 0.0
                for f in batch:
                    if weights[f] == 0.0:
                        continue
                    _, _, intrinsic, valid, target = frame_terms(f)
                    residual += float(np.sum(weights[f] * np.abs(target - intrinsic)[valid]))
                    weight_total += weights[f] * int(valid.sum())
                rms = max(float(np.sqrt(np.sum(np.abs(spectrum) ** 2))), math.sqrt(EPS))
                scale = truncation_threshold * (residual / weight_total if weight_total > 0.0 else 0.0) / rms
            maximum = max(float((np.abs(pupil) ** 2).max()), EPS)
            gradient = np.zeros_like(spectrum)
            pupil_gradient = np.zeros_like(pupil)
            source_gradient = np.zeros((frames, 2))
            source_curvature = np.zeros((frames, 2))
            source_weight = np.zeros(frames)
            active = 0
            for f in batch:
                fw = weights[f]
                if fw == 0.0:
                    continue
                active += 1
                patch, field, intrinsic, valid, target = frame_terms(f)
                frame_loss = float(np.sum(_point_loss(intrinsic, target, loss)[valid]))
                objective_sum += fw * (frame_loss / int(valid.sum()))
                weight_sum += fw
                kept = valid
                if scale is not None:
                    kept = valid & (np.abs(target - intrinsic) <= scale * np.sqrt(intrinsic))
                    rejected += int(np.sum(valid & ~kept))
                factor = np.where(kept, _descent_factor(intrinsic, target, loss), 0.0)
                projected = np.fft.fftshift(_fft_forward(field * factor))
                valid_scale = n / int(valid.sum())
                if recover_pupil:
                    object_power = max(float((np.abs(patch) ** 2).max()), EPS)
                    pupil_gradient += fw * valid_scale * np.conj(patch) * projected / (object_power + EPS)
                _insert_adjoint(gradient, model, f, np.conj(pupil) * projected / (maximum + EPS), fw * valid_scale,
                                offset_of(f))
                if recover_illumination:
                    # illumination_gradient / illumination_axis_gradient (gradient_descent.rs:1236-1345).
                    d = illumination_finite_difference
                    curvature_factor = {
                        "amplitude_mse": 0.5 / np.maximum(intrinsic, EPS),
                        "intensity_mse": np.full(intrinsic.shape, 2.0),
                        "poisson_nll": 1.0 / np.maximum(intrinsic, EPS),
                        "huber_amplitude": np.where(np.abs(factor * 2.0 * np.sqrt(np.maximum(intrinsic, EPS))) < 1.0,
                                                    0.25 / np.maximum(intrinsic, EPS), EPS),
                    }[loss]
                    for axis, shift in ((0, (d, 0.0)), (1, (0.0, d))):
                        plus, minus = offset_of(f, shift), offset_of(f, (-shift[0], -shift[1]))
                        plus_ok, minus_ok = _offset_inside(model, f, plus), _offset_inside(model, f, minus)
                        if not (plus_ok or minus_ok):
                            continue
                        if plus_ok and minus_ok:
                            derivative = (intensity_at(f, plus) - intensity_at(f, minus)) / (2.0 * d)
                        elif plus_ok:
                            derivative = (intensity_at(f, plus) - intrinsic) / d
                        else:
                            derivative = (intrinsic - intensity_at(f, minus)) / d
                        source_gradient[f, axis] += fw * float(np.sum((factor * derivative)[kept])) / int(valid.sum())
                        source_curvature[f, axis] += fw * float(np.sum((curvature_factor * derivative ** 2)[kept])) / int(valid.sum())
                    source_weight[f] += fw
            if active > 0:
                spectrum = spectrum - (object_step / active) * gradient
                if recover_pupil:
                    pupil = pupil - (pupil_step / active) * pupil_gradient
            share = len(batch) / frames
            if object_tv > 0.0:
                # apply_object_tv (gradient_descent.rs:1125-1165) on the spatial object.
                field = _fft_inverse(np.fft.ifftshift(spectrum))
                field = field - share * object_tv * _tv_gradient(field, object_tv_epsilon)
                spectrum = np.fft.fftshift(_fft_forward(field))
            if recover_pupil and pupil_smoothing > 0.0:
                pupil = pupil - share * pupil_smoothing * _smoothing_gradient(pupil)
            if recover_pupil:
                pupil = np.where(support, pupil, 0.0)
            if recover_illumination:
                # apply_illumination_update (gradient_descent.rs:1044-1089).
                for f in range(frames):
                    if source_weight[f] == 0.0:
                        continue
                    candidate = np.clip(corrections[f] - illumination_step * source_gradient[f]
                                        / (source_curvature[f] + EPS), -illumination_bounds, illumination_bounds)
                    trial = (float(model["off_row"][f]) + candidate[0], float(model["off_col"][f]) + candidate[1])
                    if _offset_inside(model, f, trial):
                        corrections[f] = candidate
        if recover_pupil and canonicalize is not None:
            spectrum, pupil = canonicalize(spectrum, pupil)
        objectives.append(objective_sum / weight_sum)
    return dict(objectives=np.array(objectives), object_spectrum=spectrum,
                object=_fft_inverse(np.fft.ifftshift(spectrum)), pupil=pupil, rejected=rejected,
                illumination_corrections=corrections)


def _schedule(name, model, data, weights, masks, background):
    """FrameSchedule::order / order_for_problem (src/reconstruction/schedule.rs:35-131):
    stable sorts by |k|, by |k| then azimuth in [0, 2 pi), or by descending
    weight * sqrt(mean(max(I - background, 0))) over unmasked pixels with
    ties in frame order and zero-weight frames last."""
    frames = data.shape[0]
    kx, ky = np.asarray(model["kx"], np.float64), np.asarray(model["ky"], np.float64)
    radius = [float(np.hypot(kx[f], ky[f])) for f in range(frames)]
    if name == "sequential":
        return list(range(frames))
    if name == "brightfield_first":
        return sorted(range(frames), key=lambda f: radius[f])
    if name == "spiral_out":
        return sorted(range(frames), key=lambda f: (radius[f], math.atan2(ky[f], kx[f]) % math.tau))
    scores = []
    for f in range(frames):
        valid = np.ones(data.shape[1:], bool) if masks is None else masks[f] != 0
        if weights[f] == 0.0 or not valid.any():
            scores.append(-math.inf)
            continue
        signal = float(np.sum(np.maximum(data[f] - background[f], 0.0)[valid]))
        scores.append(weights[f] * math.sqrt(signal / int(valid.sum())))
    return sorted(range(frames), key=lambda f: (-scores[f], f))


def _direct_model():
    # tests/common/mod.rs:49-81: 8x8 detector, 16x16 grid, unit pupil, five integer crops.
    shifts = [(-3, 0), (0, -3), (0, 0), (0, 3), (3, 0)]
    return dict(h=8, w=8, mh=16, mw=16, start_row=np.array([4 + r for c, r in shifts], np.int64),
                start_col=np.array([4 + c for c, r in shifts], np.int64), off_row=np.zeros(5), off_col=np.zeros(5),
                pupil=np.ones((8, 8), np.complex128), support=np.ones((8, 8), np.uint8))


def _compare(want, got, iterations, rtol=1e-9):
    assert np.allclose(got["objectives"], want["objectives"][:iterations], rtol=rtol, atol=0.0)
    scale = np.abs(want["object"]).max()
    assert np.abs(got["object"] - want["object"]).max() <= rtol * scale
    assert np.abs(got["object_spectrum"] - want["object_spectrum"]).max() <= rtol * np.abs(want["object_spectrum"]).max()


_ORACLE_OPTIONS = {"epry": dict(recover_pupil=False)}


@pytest.mark.parametrize("algorithm", ["ap", "fpie", "mpie", "epry"])
def test_direct_model_trajectories_agree(oracle_module, algorithm):
    model = _direct_model()
    rng = np.random.default_rng(21)
    truth = np.exp(1j * 0.4 * rng.standard_normal((16, 16))) * (0.7 + 0.3 * rng.random((16, 16)))
    data = oracle.forward_stack(oracle.Problem(model, None), oracle.object_spectrum(truth))
    iterations = 40 if algorithm == "mpie" else 6  # mPIE: 200 frame updates, six momentum events
    want = oracle.run(oracle.Problem(model, data), algorithm, iterations=iterations, **_ORACLE_OPTIONS.get(algorithm, {}))
    _compare(want, restated_run(model, data, algorithm, iterations), iterations)


@pytest.mark.parametrize("algorithm", ["ap", "fpie", "mpie", "epry"])
@pytest.mark.parametrize("loss", ["amplitude_mse", "intensity_mse", "poisson_nll", "huber_amplitude"])
def test_subpixel_masked_weighted_trajectories_agree(oracle_module, native_library, algorithm, loss):
    """A compiled 5 x 5 planar tile (fractional crop offsets) with an
    apodized, aberrated pupil (so |P|^2 varies and the local and rPIE
    denominators differ), Poisson counts with gains and a per-frame
    background, masked pixels and one zero-weight frame, under each loss."""
    import fpm_rs as fpm

    _, model = helpers.planar_model(fpm, 5, 32)
    assert np.any(np.abs(model["off_row"]) > 1e-12) or np.any(np.abs(model["off_col"]) > 1e-12)
    support = model["support"].astype(bool)
    apodized = W.zernike_pupil(model["support"], 3) * np.where(support, 0.4 + 0.6 * np.random.default_rng(8).random(support.shape), 0.0)
    model = dict(model, pupil=apodized)
    truth = W.smooth_random_object((model["mh"], model["mw"]), 5)
    intensity = oracle.forward_stack(oracle.Problem(model, None), oracle.object_spectrum(truth))
    frames = intensity.shape[0]
    rng = np.random.default_rng(6)
    gains = rng.uniform(200.0, 400.0, frames)
    background = rng.uniform(0.0, 3.0, (frames, 32, 32))
    data = rng.poisson(intensity * gains[:, None, None]) + background
    masks = (rng.random(data.shape) > 0.1).astype(np.uint8)
    weights = np.ones(frames)
    weights[7] = 0.0
    problem = oracle.Problem(model, data, gains=gains, background=background, masks=masks, weights=weights)
    want = oracle.run(problem, algorithm, iterations=3, loss_type=loss, **_ORACLE_OPTIONS.get(algorithm, {}))
    got = restated_run(model, data, algorithm, 3, loss=loss, weights=weights, masks=masks, gains=gains,
                       background=background)
    _compare(want, got, 3)


@pytest.mark.parametrize("recover", ["gains", "background", "both"])
def test_epry_gain_and_background_recovery_trajectories_agree(oracle_module, native_library, recover):
    """EPRY with a fixed pupil recovering frame gains and per-frame
    backgrounds that the model gets wrong, on the same compiled tile."""
    import fpm_rs as fpm

    _, model = helpers.planar_model(fpm, 5, 32)
    truth = W.smooth_random_object((model["mh"], model["mw"]), 7)
    intensity = oracle.forward_stack(oracle.Problem(model, None), oracle.object_spectrum(truth))
    frames = intensity.shape[0]
    rng = np.random.default_rng(12)
    true_gains = rng.uniform(200.0, 400.0, frames)
    true_background = rng.uniform(2.0, 6.0, frames)[:, None, None] * np.ones((1, 32, 32))
    data = rng.poisson(intensity * true_gains[:, None, None]) + true_background
    masks = (rng.random(data.shape) > 0.1).astype(np.uint8)
    model_gains = np.full(frames, 300.0)
    model_background = np.full((frames, 32, 32), 4.0)
    gains_on, background_on = recover in ("gains", "both"), recover in ("background", "both")
    problem = oracle.Problem(model, data, gains=model_gains, background=model_background, masks=masks)
    want = oracle.run(problem, "epry", iterations=3, recover_pupil=False, recover_gains=gains_on,
                      recover_background=background_on)
    got = restated_run(model, data, "epry", 3, masks=masks, gains=model_gains, background=model_background,
                       recover_gains=gains_on, recover_background=background_on)
    _compare(want, got, 3)
    if gains_on:
        assert np.allclose(got["frame_gains"], want["frame_gains"], rtol=1e-9, atol=0.0)
        assert not np.allclose(got["frame_gains"], model_gains)
    if background_on:
        assert np.allclose(got["background"], want["background"], rtol=1e-9, atol=0.0)
        assert not np.allclose(got["background"], model_background)


@pytest.mark.parametrize("batch_size", [1, 4, 9])
@pytest.mark.parametrize("loss", ["amplitude_mse", "intensity_mse", "poisson_nll", "huber_amplitude"])
def test_gradient_descent_trajectories_agree(oracle_module, native_library, batch_size, loss):
    """Gradient descent on the same compiled tile, apodized pupil, gains,
    background, masks and a zero-weight frame, in mini-batches. The Poisson
    descent factor 1 - I / max(|psi|^2, eps) reaches about 1e8 on dark fringe
    pixels, which magnifies last-bit differences between the two FFTs: with
    one frame per step it is compared over two passes at 1e-5 (the
    objectives still agree to 1e-9); every other case over three passes at
    1e-9."""
    import fpm_rs as fpm

    _, model = helpers.planar_model(fpm, 5, 32)
    support = model["support"].astype(bool)
    model = dict(model, pupil=W.zernike_pupil(model["support"], 4)
                 * np.where(support, 0.4 + 0.6 * np.random.default_rng(9).random(support.shape), 0.0))
    truth = W.smooth_random_object((model["mh"], model["mw"]), 6)
    intensity = oracle.forward_stack(oracle.Problem(model, None), oracle.object_spectrum(truth))
    frames = intensity.shape[0]
    rng = np.random.default_rng(10)
    gains = rng.uniform(200.0, 400.0, frames)
    background = rng.uniform(0.0, 3.0, (frames, 32, 32))
    data = rng.poisson(intensity * gains[:, None, None]) + background
    masks = (rng.random(data.shape) > 0.1).astype(np.uint8)
    weights = np.ones(frames)
    weights[3] = 0.0
    problem = oracle.Problem(model, data, gains=gains, background=background, masks=masks, weights=weights)
    sensitive = loss == "poisson_nll" and batch_size == 1
    iterations = 2 if sensitive else 3
    want = oracle.run(problem, "gd", iterations=iterations, loss_type=loss, batch_size=batch_size)
    got = restated_gd(model, data, iterations, batch_size, loss=loss, weights=weights, masks=masks, gains=gains,
                      background=background)
    _compare(want, got, iterations, rtol=1e-5 if sensitive else 1e-9)
    assert np.allclose(got["objectives"], want["objectives"], rtol=1e-9, atol=0.0)


@pytest.mark.parametrize("schedule", ["brightfield_first", "spiral_out", "snr_weighted"])
def test_schedules_order_frames_as_the_reference(oracle_module, native_library, schedule):
    """The same tile under each deterministic schedule, with mPIE (frame by
    frame) and gradient descent (batches of four taken from the ordered
    frames), against the oracle's runs."""
    import fpm_rs as fpm

    _, model = helpers.planar_model(fpm, 5, 32)
    truth = W.smooth_random_object((model["mh"], model["mw"]), 8)
    intensity = oracle.forward_stack(oracle.Problem(model, None), oracle.object_spectrum(truth))
    frames = intensity.shape[0]
    rng = np.random.default_rng(13)
    gains = np.full(frames, 300.0)
    background = rng.uniform(0.0, 3.0, (frames, 32, 32))
    data = rng.poisson(intensity * gains[:, None, None]) + background
    masks = (rng.random(data.shape) > 0.1).astype(np.uint8)
    weights = rng.uniform(0.5, 1.5, frames)
    weights[11] = 0.0
    # Frames 2 and 5 score alike, so the SNR order must break their tie by index.
    data[5], masks[5], background[5], weights[5] = data[2], masks[2], background[2], weights[2]
    order = _schedule(schedule, model, data, weights, masks, background)
    assert sorted(order) == list(range(frames)) and order != list(range(frames))
    if schedule == "snr_weighted":
        assert order.index(2) + 1 == order.index(5) and order[-1] == 11
    problem = oracle.Problem(model, data, gains=gains, background=background, masks=masks, weights=weights)
    want = oracle.run(problem, "mpie", iterations=2, schedule=schedule)
    got = restated_run(model, data, "mpie", 2, weights=weights, masks=masks, gains=gains, background=background,
                       order=order)
    _compare(want, got, 2)
    want = oracle.run(problem, "gd", iterations=2, schedule=schedule, batch_size=4)
    got = restated_gd(model, data, 2, 4, weights=weights, masks=masks, gains=gains, background=background,
                      order=order)
    _compare(want, got, 2)


def restated_spectral(channels, frames, data, iterations, *, shared=False, weights=None, masks=None,
                      loss="amplitude_mse", object_step=1.0, initial_spectra=None):
    """Spectral alternating projection (src/algorithms/spectral.rs:182-271,
    src/reconstruction/spectral.rs:127-230 and :271-331): each exposure's
    modes are evaluated from the pre-exposure objects, share one projection
    ratio against gain * sum_k w_k |psi_k|^2 + background, and each adds its
    local-denominator update scaled by w_k / sum w."""
    exposures = len(frames)
    weights = np.ones(exposures) if weights is None else np.asarray(weights, np.float64)
    count = 1 if shared else len(channels)
    index = (lambda c: 0) if shared else (lambda c: c)
    fg = [np.asarray(ch.get("frame_gains", np.ones(len(ch["start_row"]))), np.float64) for ch in channels]
    h, w, mh, mw = channels[0]["h"], channels[0]["w"], channels[0]["mh"], channels[0]["mw"]
    spectra = []
    for o in range(count):
        average, weight = np.zeros((h, w)), np.zeros((h, w))
        total_amplitude = total_weight = 0.0
        for e, (gain, background, contributions) in enumerate(frames):
            if not any(index(c) == o for c, _, _ in contributions) or weights[e] == 0.0:
                continue
            g = sum(s * fg[c][l] for c, l, s in contributions) * gain
            valid = np.ones((h, w), bool) if masks is None else masks[e] != 0
            amplitude = np.sqrt(np.maximum((data[e] - background) / g, 0.0))
            average[valid] += weights[e] * amplitude[valid]
            weight[valid] += weights[e]
            total_amplitude += float(np.sum(weights[e] * amplitude[valid]))
            total_weight += weights[e] * int(valid.sum())
        average = np.where(weight > 0.0, average / np.where(weight > 0.0, weight, 1.0), total_amplitude / total_weight)
        obj = average[((np.arange(mh) * h) // mh)[:, None], ((np.arange(mw) * w) // mw)[None, :]].astype(np.complex128)
        spectra.append(np.fft.fftshift(_fft_forward(obj)))
    if initial_spectra is not None:
        spectra = [np.array(x, np.complex128) for x in initial_spectra]
    objectives = []
    for _ in range(iterations):
        objective_sum = weight_sum = 0.0
        for e, (gain, background, contributions) in enumerate(frames):
            fw = weights[e]
            if fw == 0.0:
                continue
            separate = len(contributions) == 1
            effective_gain = gain * (contributions[0][2] * fg[contributions[0][0]][contributions[0][1]] if separate else 1.0)
            modes, predicted = [], np.zeros((h, w))
            for c, l, s in contributions:
                mode_weight = 1.0 if separate else s * fg[c][l]
                exit_wave = _extract(spectra[index(c)], channels[c], l) * channels[c]["pupil"]
                psi = _fft_inverse(np.fft.ifftshift(exit_wave))
                predicted = predicted + mode_weight * np.abs(psi) ** 2
                modes.append((c, l, mode_weight, psi, exit_wave))
            mode_sum = sum(m[2] for m in modes)
            valid = np.ones((h, w), bool) if masks is None else masks[e] != 0
            loss_value = float(np.sum(_point_loss(effective_gain * predicted + background, data[e], loss)[valid]))
            objective_sum += fw * (loss_value / int(valid.sum()))
            weight_sum += fw
            target = np.maximum((data[e] - background) / effective_gain, 0.0)
            bright = predicted > EPS
            ratio = np.sqrt(target / np.where(bright, predicted, 1.0))
            dark = np.sqrt(target / mode_sum)
            for c, l, mode_weight, psi, exit_wave in modes:
                projected = np.where(valid, np.where(bright, psi * ratio, dark + 0j), psi)
                centred = np.fft.fftshift(_fft_forward(projected))
                pupil = channels[c]["pupil"]
                update = np.conj(pupil) * (centred - exit_wave) / (np.abs(pupil) ** 2 + EPS)
                _insert_adjoint(spectra[index(c)], channels[c], l, update, fw * object_step * (mode_weight / mode_sum))
        objectives.append(objective_sum / weight_sum)
    return dict(objectives=np.array(objectives), spectra=np.stack(spectra),
                objects=np.stack([_fft_inverse(np.fft.ifftshift(s)) for s in spectra]))


@pytest.mark.parametrize("plan", ["separate", "multiplexed_shared"])
def test_spectral_trajectories_agree(oracle_module, plan):
    """Three channels compiled on one grid: separate exposures with
    independent objects, or every exposure mixing all three channels into
    one shared object; frame and exposure gains, backgrounds, masks and a
    zero-weight exposure."""
    import spectral_cases as sc

    gains = [np.random.default_rng(14 + c).uniform(0.8, 1.2, len(sc.DIRECTIONS)) for c in range(3)]
    channels = [dict(ch, frame_gains=g) for ch, g in zip(sc.compile_channels(3, image_shape=(32, 32)), gains)]
    shared = plan == "multiplexed_shared"
    if shared:
        frames = [(1.7, 0.3, [(c, l, 0.4 + 0.2 * c) for c in range(3)]) for l in range(len(sc.DIRECTIONS))]
    else:
        frames = [(1.0 + 0.1 * l, 0.2 * c, [(c, l, 1.0)]) for c in range(3) for l in range(len(sc.DIRECTIONS))]
    truth = sc.truth_objects((channels[0]["mh"], channels[0]["mw"]), 1 if shared else 3)
    problem = oracle.SpectralProblem(channels, frames, shared_object=shared)
    intensity = oracle.spectral_forward(problem, sc.spectra_of(truth))
    rng = np.random.default_rng(15)
    data = rng.poisson(intensity * 500.0) / 500.0
    masks = (rng.random(data.shape) > 0.1).astype(np.uint8)
    weights = np.ones(len(frames))
    weights[1] = 0.0
    want = oracle.spectral_run(oracle.SpectralProblem(channels, frames, data, shared_object=shared, weights=weights,
                                                      masks=masks), iterations=4)
    got = restated_spectral(channels, frames, data, 4, shared=shared, weights=weights, masks=masks)
    assert np.allclose(got["objectives"], want["objectives"], rtol=1e-9, atol=0.0)
    assert np.abs(got["spectra"] - want["spectra"]).max() <= 1e-9 * np.abs(want["spectra"]).max()
    assert np.abs(got["objects"] - want["objects"]).max() <= 1e-9 * np.abs(want["objects"]).max()


def _zero_stencil(spectrum, model, source):
    """The spectrum with `source`'s whole crop stencil set to zero, so that
    frame's field is exactly zero and every pixel takes the dark branch."""
    out = np.array(spectrum, np.complex128)
    taps, h, w = _stencil(model, source)
    for r, c, _ in taps:
        out[r:r + h, c:c + w] = 0.0
    return out


@pytest.mark.parametrize("algorithm", ["ap", "mpie"])
def test_dark_frames_take_the_fallback_amplitude(oracle_module, native_library, algorithm):
    """A start whose spectrum vanishes on frame 0's stencil: every pixel of
    that frame is dark (|psi|^2 <= eps), so its projection is the fallback
    sqrt(target) (common.rs:184-190) and its update is still non-zero."""
    import fpm_rs as fpm

    _, model = helpers.planar_model(fpm, 5, 32)
    truth = W.smooth_random_object((model["mh"], model["mw"]), 9)
    spectrum = oracle.object_spectrum(truth)
    data = oracle.forward_stack(oracle.Problem(model, None), spectrum)
    start = _zero_stencil(spectrum, model, 0)
    want = oracle.run(oracle.Problem(model, data), algorithm, iterations=2, initial_spectrum=start)
    got = restated_run(model, data, algorithm, 2, initial_spectrum=start)
    _compare(want, got, 2)


def test_dark_spectral_exposure_takes_the_fallback_over_the_mode_weights(oracle_module):
    """The same for a multiplexed exposure on a shared object: its fallback
    amplitude is sqrt(target / sum of mode weights) (spectral.rs:221-225)."""
    import spectral_cases as sc

    channels = sc.compile_channels(3, image_shape=(32, 32))
    frames = [(1.7, 0.3, [(c, l, 0.4 + 0.2 * c) for c in range(3)]) for l in range(len(sc.DIRECTIONS))]
    truth = sc.truth_objects((channels[0]["mh"], channels[0]["mw"]), 1)
    spectra = sc.spectra_of(truth)
    data = oracle.spectral_forward(oracle.SpectralProblem(channels, frames, shared_object=True), spectra)
    start = spectra[0]
    for c in range(3):
        start = _zero_stencil(start, channels[c], 0)
    want = oracle.spectral_run(oracle.SpectralProblem(channels, frames, data, shared_object=True), iterations=2,
                               initial_spectra=start[None])
    got = restated_spectral(channels, frames, data, 2, shared=True, initial_spectra=start[None])
    assert np.allclose(got["objectives"], want["objectives"], rtol=1e-9, atol=0.0)
    assert np.abs(got["spectra"] - want["spectra"]).max() <= 1e-9 * np.abs(want["spectra"]).max()


def test_adaptive_ap_step_controller_trajectory_agrees(oracle_module, native_library):
    """Adaptive AP with a threshold that most passes miss, so the step halves
    down to its floor, on the compiled tile with an apodized pupil."""
    import fpm_rs as fpm

    _, model = helpers.planar_model(fpm, 5, 32)
    support = model["support"].astype(bool)
    model = dict(model, pupil=np.where(support, 0.5 + 0.5 * np.random.default_rng(16).random(support.shape), 0.0)
                 + 0j)
    truth = W.smooth_random_object((model["mh"], model["mw"]), 10)
    data = oracle.forward_stack(oracle.Problem(model, None), oracle.object_spectrum(truth))
    options = dict(progress_threshold=0.6, reduction_factor=0.5, minimum_object_step=0.2)
    want = oracle.run(oracle.Problem(model, data), "adaptive_ap", iterations=8, **options)
    got = restated_run(model, data, "adaptive_ap", 8, **options)
    _compare(want, got, 8)
    assert np.array_equal(got["object_steps"], want["object_steps"][:8])
    assert list(got["object_steps"]) == [1.0, 1.0, 1.0, 1.0, 0.5, 0.25, 0.2, 0.2]


@pytest.mark.parametrize("variant", ["pupil_recovery", "poisson_truncation"])
def test_gradient_descent_pupil_recovery_and_truncation_agree(oracle_module, native_library, variant):
    """GD recovering an aberrated pupil inside its support, and GD under the
    Poisson loss with truncation that rejects outliers planted in the data,
    in batches of four with masked pixels, against the oracle."""
    import fpm_rs as fpm

    _, model = helpers.planar_model(fpm, 5, 32)
    true_pupil = W.zernike_pupil(model["support"], 5)
    truth = W.smooth_random_object((model["mh"], model["mw"]), 11)
    intensity = oracle.forward_stack(oracle.Problem(dict(model, pupil=true_pupil), None), oracle.object_spectrum(truth))
    rng = np.random.default_rng(17)
    data = rng.poisson(intensity * 300.0) / 300.0
    data.reshape(data.shape[0], -1)[:, ::97] *= 20.0  # outliers
    masks = (rng.random(data.shape) > 0.1).astype(np.uint8)
    kw = (dict(recover_pupil=True, pupil_step=0.05) if variant == "pupil_recovery"
          else dict(loss="poisson_nll", truncation_threshold=3.0))
    oracle_kw = (dict(recover_pupil=True, pupil_step=0.05) if variant == "pupil_recovery"
                 else dict(loss_type="poisson_nll", poisson_truncation_threshold=3.0))
    want = oracle.run(oracle.Problem(model, data, masks=masks), "gd", iterations=3, batch_size=4, **oracle_kw)
    gauge = lambda spectrum, pupil: oracle.canonicalize(oracle.Problem(model, data, masks=masks), spectrum, pupil)
    got = restated_gd(model, data, 3, 4, masks=masks, canonicalize=gauge, **kw)
    _compare(want, got, 3)
    if variant == "pupil_recovery":
        assert np.abs(got["pupil"] - want["pupil"]).max() <= 1e-9 * np.abs(want["pupil"]).max()
        assert not np.allclose(got["pupil"], model["pupil"])
    else:
        assert got["rejected"] > 0


def test_epry_pupil_recovery_trajectory_agrees(oracle_module, native_library):
    """EPRY recovering an aberrated pupil (apodized start) with masked
    pixels, the gauge step through the oracle's canonicalisation."""
    import fpm_rs as fpm

    _, model = helpers.planar_model(fpm, 5, 32)
    true_pupil = W.zernike_pupil(model["support"], 6)
    truth = W.smooth_random_object((model["mh"], model["mw"]), 12)
    intensity = oracle.forward_stack(oracle.Problem(dict(model, pupil=true_pupil), None), oracle.object_spectrum(truth))
    rng = np.random.default_rng(18)
    data = rng.poisson(intensity * 300.0) / 300.0
    masks = (rng.random(data.shape) > 0.1).astype(np.uint8)
    problem = oracle.Problem(model, data, masks=masks)
    want = oracle.run(problem, "epry", iterations=3, recover_pupil=True)
    got = restated_run(model, data, "epry", 3, masks=masks, recover_pupil=True,
                       canonicalize=lambda s, p: oracle.canonicalize(problem, s, p))
    _compare(want, got, 3)
    assert np.abs(got["pupil"] - want["pupil"]).max() <= 1e-9 * np.abs(want["pupil"]).max()
    assert not np.allclose(got["pupil"], model["pupil"])


@pytest.mark.parametrize("variant", ["object_tv", "pupil_smoothing"])
def test_gradient_descent_regularisers_agree(oracle_module, native_library, variant):
    """GD with the object TV step, or with pupil recovery and pupil
    smoothing, in batches of four with masked pixels and a zero-weight frame
    (whose batch still counts it in the regulariser share)."""
    import fpm_rs as fpm

    _, model = helpers.planar_model(fpm, 5, 32)
    truth = W.smooth_random_object((model["mh"], model["mw"]), 13)
    true_pupil = W.zernike_pupil(model["support"], 7)
    intensity = oracle.forward_stack(oracle.Problem(dict(model, pupil=true_pupil), None), oracle.object_spectrum(truth))
    rng = np.random.default_rng(19)
    data = rng.poisson(intensity * 300.0) / 300.0
    masks = (rng.random(data.shape) > 0.1).astype(np.uint8)
    weights = np.ones(data.shape[0])
    weights[6] = 0.0
    problem = oracle.Problem(model, data, masks=masks, weights=weights)
    if variant == "object_tv":
        kw = dict(object_tv=0.05, object_tv_epsilon=1e-3)
        oracle_kw = dict(object_tv_weight=0.05, object_tv_epsilon=1e-3)
    else:
        kw = dict(recover_pupil=True, pupil_step=0.05, pupil_smoothing=0.02)
        oracle_kw = dict(recover_pupil=True, pupil_step=0.05, pupil_smoothing_weight=0.02)
    want = oracle.run(problem, "gd", iterations=3, batch_size=4, **oracle_kw)
    got = restated_gd(model, data, 3, 4, masks=masks, weights=weights,
                      canonicalize=lambda s, p: oracle.canonicalize(problem, s, p), **kw)
    _compare(want, got, 3)
    if variant == "pupil_smoothing":
        assert np.abs(got["pupil"] - want["pupil"]).max() <= 1e-9 * np.abs(want["pupil"]).max()


@pytest.mark.parametrize("batch_size,loss", [(1, "amplitude_mse"), (4, "intensity_mse"), (1, "huber_amplitude"),
                                             (4, "poisson_nll")])
def test_gradient_descent_illumination_recovery_agrees(oracle_module, native_library, batch_size, loss):
    """GD recovering per-source offsets from data simulated with shifted
    sources, masked pixels, under four losses."""
    import fpm_rs as fpm

    _, model = helpers.planar_model(fpm, 5, 32)
    shifted = dict(model, off_row=model["off_row"] + 0.3 * np.sin(np.arange(25)),
                   off_col=model["off_col"] - 0.25 * np.cos(np.arange(25)))
    truth = W.smooth_random_object((model["mh"], model["mw"]), 14)
    intensity = oracle.forward_stack(oracle.Problem(shifted, None), oracle.object_spectrum(truth))
    rng = np.random.default_rng(20)
    data = rng.poisson(intensity * 300.0) / 300.0
    masks = (rng.random(data.shape) > 0.1).astype(np.uint8)
    problem = oracle.Problem(model, data, masks=masks)
    want = oracle.run(problem, "gd", iterations=3, batch_size=batch_size, loss_type=loss, recover_illumination=True)
    got = restated_gd(model, data, 3, batch_size, loss=loss, masks=masks, recover_illumination=True)
    _compare(want, got, 3)
    assert np.allclose(got["illumination_corrections"], want["illumination_corrections"], rtol=1e-9, atol=1e-12)
    assert np.abs(got["illumination_corrections"]).max() > 1e-3
