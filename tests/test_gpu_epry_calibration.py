"""EPRY frame-gain and background recovery on the device against the FP64
oracle (update_gain / update_background, src/algorithms/common.rs:390-489).

Data: the FP64 forward stack of a smooth random object, with per-frame
gains and per-frame constant backgrounds that the reconstruction model does
not know; Poisson noise. Tolerances: object NRMSE <= 1e-4; recovered gains
and backgrounds within 1e-4 relative (of the largest value); objectives to
1e-4 relative. The amplitude form (no model background) reads intensities
as g0 a^2 from the stored FP32 amplitudes, so its recovered values carry
that rounding too.
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


def _data(fpm, side, n, seed, gain_spread=0.3, background=None, pupil_seed=None):
    """Counts with hidden per-frame gain factors and backgrounds."""
    model, omodel = helpers.planar_model(fpm, side, n)
    truth = W.smooth_random_object(model.reconstruction_shape, seed)
    sim = dict(omodel)
    if pupil_seed is not None:
        sim["pupil"] = W.zernike_pupil(omodel["support"], pupil_seed)
    intensity = oracle.forward_stack(oracle.Problem(sim, None), oracle.object_spectrum(truth), workers=8)
    counts, scale = W.poisson_counts(intensity, 1e4, seed + 1)
    frames = counts.shape[0]
    rng = np.random.default_rng(seed + 2)
    factors = 1.0 + gain_spread * (rng.random(frames) - 0.5)
    data = counts * factors[:, None, None]
    if background is not None:
        data = data + background[:, None, None]
    gains = np.full(frames, scale)
    return model._replace(frame_gains=gains), omodel, data, gains


def _close(got, want, rtol):
    got, want = np.asarray(got), np.asarray(want)
    assert got.shape == want.shape
    scale = max(np.abs(want).max(), 1e-300)
    assert np.abs(got - want).max() <= rtol * scale, (np.abs(got - want).max(), scale)


def _objectives_close(gpu, cpu, rtol=1e-4):
    gpu, cpu = np.asarray(gpu), np.asarray(cpu)
    assert np.all(np.abs(gpu - cpu) <= rtol * np.abs(cpu) + 1e-12), (gpu, cpu)


@pytest.mark.parametrize("n,side", [(32, 3), (64, 5)])
def test_frame_gain_recovery_matches_oracle(fpm, n, side):
    model, omodel, data, gains = _data(fpm, side, n, seed=60)
    kw = dict(iterations=4, recover_pupil=False)
    got = fpm.Epry(**kw, recover_frame_gains=True, gain_step=0.5).run(fpm.ReconstructionProblem(data, model))
    want = oracle.run(oracle.Problem(omodel, data, gains=gains), "epry", **kw, recover_gains=True, gain_step=0.5)
    assert oracle.complex_nrmse(want["object"], got.object) <= NRMSE
    _close(got.recovered_frame_gains, want["frame_gains"], 1e-4)
    _objectives_close([t[1] for t in got.trace], want["objectives"])
    # The gains moved: recovery did something.
    assert np.abs(np.asarray(got.recovered_frame_gains) - gains).max() > 1e-3 * gains.max()


def test_background_recovery_matches_oracle(fpm):
    rng = np.random.default_rng(7)
    model, omodel, data, gains = _data(fpm, 5, 64, seed=61, gain_spread=0.0,
                                       background=rng.uniform(0.0, 40.0, 25))
    kw = dict(iterations=3, recover_pupil=False)
    algo = fpm.Epry(**kw, recover_background=True, background_step=0.5, background_bounds=(-100.0, 100.0))
    got = algo.run(fpm.ReconstructionProblem(data, model))
    want = oracle.run(oracle.Problem(omodel, data, gains=gains), "epry", **kw, recover_background=True,
                      background_step=0.5, background_min=-100.0, background_max=100.0)
    assert oracle.complex_nrmse(want["object"], got.object) <= NRMSE
    _close(got.recovered_background, want["background"], 1e-4)
    _objectives_close([t[1] for t in got.trace], want["objectives"])


def test_gain_and_background_with_model_background_and_pupil_recovery(fpm):
    """Both recoveries with a model background (raw measurement form, the
    state background starting from the model's) and pupil recovery at 128
    points, with masked pixels."""
    rng = np.random.default_rng(8)
    model, omodel, data, gains = _data(fpm, 5, 128, seed=62, background=rng.uniform(5.0, 20.0, 25), pupil_seed=11)
    background = np.full(128 * 128, 6.0)
    model = model._replace(background=background)
    masks = (np.random.default_rng(9).random(data.shape) > 0.1).astype(np.uint8)
    kw = dict(iterations=3)
    algo = fpm.Epry(**kw, recover_frame_gains=True, recover_background=True, background_bounds=(0.0, 1e3))
    got = algo.run(fpm.ReconstructionProblem(data, model, masks=masks))
    want = oracle.run(oracle.Problem(omodel, data, gains=gains, background=background, masks=masks), "epry", **kw,
                      recover_gains=True, recover_background=True, background_min=0.0, background_max=1e3)
    assert oracle.complex_nrmse(want["object"], got.object) <= NRMSE
    assert oracle.complex_nrmse(want["pupil"], got.recovered_pupil) <= NRMSE
    _close(got.recovered_frame_gains, want["frame_gains"], 1e-4)
    _close(got.recovered_background, want["background"], 1e-4)
    _objectives_close([t[1] for t in got.trace], want["objectives"])


def test_recovery_parameters_are_validated(fpm):
    model, omodel, data, gains = _data(fpm, 3, 32, seed=63)
    problem = fpm.ReconstructionProblem(data, model)
    for bad in (dict(recover_frame_gains=True, gain_step=1.5), dict(recover_frame_gains=True, gain_bounds=(2.0, 1.0)),
                dict(recover_background=True, background_step=-0.1),
                dict(recover_background=True, background_bounds=(1.0, 1.0))):
        with pytest.raises(fpm.InvalidParameterError):
            fpm.Epry(iterations=1, **bad).run(problem)
