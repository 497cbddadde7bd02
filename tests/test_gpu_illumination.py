"""GPU parity of gradient-descent illumination (source-offset) recovery
against the FP64 oracle's restatement of GradientDescent with
recover_illumination (src/algorithms/gradient_descent.rs:528-613,
1044-1089, 1236-1368).

The data are simulated with the centre LED displaced by (0.3, -0.2)
subpixels and reconstructed with the nominal model. The device evaluates the
finite differences in FP32 from the batch-start state, so the recovered
corrections agree with the oracle's to 2e-3 subpixels, objects to a complex
NRMSE of 1e-3 and objectives to 1e-3 relative (the FP32 engine alone holds
1e-4 on the same runs).
"""

from __future__ import annotations

import numpy as np
import pytest

import helpers
import oracle
import workloads as W

pytestmark = pytest.mark.gpu

CORRECTION_TOL = 2e-3
NRMSE = 1e-3


@pytest.fixture(scope="module")
def fpm(native_library):
    import fpm_rs

    return fpm_rs


def _case(fpm, side, n, seed):
    model, omodel = helpers.planar_model(fpm, side, n)
    truth = W.smooth_random_object(model.reconstruction_shape, seed)
    sim = dict(omodel, off_row=omodel["off_row"].copy(), off_col=omodel["off_col"].copy())
    centre = model.frame_count // 2
    sim["off_row"][centre] += 0.3
    sim["off_col"][centre] -= 0.2
    data = oracle.forward_stack(oracle.Problem(sim, None), oracle.object_spectrum(truth), workers=8)
    return model, omodel, data


def _compare(fpm, model, omodel, data, *, weights=None, masks=None, **kw):
    problem = fpm.ReconstructionProblem(data, model, frame_weights=weights, masks=masks)
    result = fpm.GradientDescent(recover_illumination=True, **kw).run(problem)
    expected = oracle.run(oracle.Problem(omodel, data, weights=weights, masks=masks), "gd",
                          recover_illumination=True, **kw)
    got, want = result.calibrated_illumination, expected["illumination_corrections"]
    assert got is not None and got.shape == (model.frame_count, 2)
    assert np.abs(want).max() > 0.01  # the recovery moved
    err = np.abs(got - want).max()
    assert err <= CORRECTION_TOL, (err, got, want)
    nrmse = oracle.complex_nrmse(expected["object"], result.object)
    assert nrmse <= NRMSE, nrmse
    gpu = np.array([t[1] for t in result.trace])
    assert np.all(np.abs(gpu - expected["objectives"]) <= 1e-3 * np.abs(expected["objectives"]) + 1e-12), (
        gpu, expected["objectives"])
    return result, expected


@pytest.mark.parametrize("n,side,batch,loss", [(32, 3, 1, "amplitude_mse"), (32, 5, 4, "poisson_nll"),
                                               (64, 3, 9, "intensity_mse"), (128, 3, 1, "huber_amplitude"),
                                               (256, 3, 3, "amplitude_mse")])
def test_illumination_recovery_matches_oracle(fpm, n, side, batch, loss):
    model, omodel, data = _case(fpm, side, n, seed=61)
    _compare(fpm, model, omodel, data, iterations=4, batch_size=batch, loss_type=loss, illumination_step=0.5,
             illumination_bounds=0.5)


def test_illumination_recovery_with_masks_weights_and_tv(fpm):
    model, omodel, data = _case(fpm, 5, 32, seed=62)
    rng = np.random.default_rng(63)
    masks = (rng.random(data.shape) > 0.05).astype(np.uint8)
    weights = np.ones(model.frame_count)
    weights[2] = 0.0
    weights[6] = 0.5
    # The Python API names the TV weight object_tv; the oracle object_tv_weight.
    problem = fpm.ReconstructionProblem(data, model, frame_weights=weights, masks=masks)
    kw = dict(iterations=3, batch_size=2, illumination_step=0.5, illumination_bounds=0.5)
    result = fpm.GradientDescent(recover_illumination=True, object_tv=0.002, **kw).run(problem)
    expected = oracle.run(oracle.Problem(omodel, data, weights=weights, masks=masks), "gd", recover_illumination=True,
                          object_tv_weight=0.002, **kw)
    got, want = result.calibrated_illumination, expected["illumination_corrections"]
    assert np.abs(got - want).max() <= CORRECTION_TOL, (got, want)
    assert np.all(got[2] == 0.0)  # a zero-weight frame keeps its offset
    assert oracle.complex_nrmse(expected["object"], result.object) <= NRMSE


def test_illumination_run_leaves_the_problem_unchanged_and_batches_match(fpm):
    # The recovered offsets live in the run's own frame constants: a later
    # plain run of the same resident problem equals one of a fresh problem,
    # and a batched illumination run equals single runs bitwise.
    model, omodel, data = _case(fpm, 3, 32, seed=64)
    problem = fpm.ReconstructionProblem(data, model)
    algo = fpm.GradientDescent(iterations=3, recover_illumination=True, illumination_step=0.5)
    first = algo.run(problem)
    plain = fpm.GradientDescent(iterations=3).run(problem)
    fresh = fpm.GradientDescent(iterations=3).run(fpm.ReconstructionProblem(data, model))
    np.testing.assert_array_equal(plain.object_spectrum, fresh.object_spectrum)
    other_model, _, other_data = _case(fpm, 3, 32, seed=65)
    other = fpm.ReconstructionProblem(other_data, other_model)
    batch = fpm.run_batch(algo, [fpm.ReconstructionProblem(data, model), other])
    np.testing.assert_array_equal(batch[0].object_spectrum, first.object_spectrum)
    np.testing.assert_array_equal(batch[0].calibrated_illumination, first.calibrated_illumination)
    alone = algo.run(other)
    np.testing.assert_array_equal(batch[1].calibrated_illumination, alone.calibrated_illumination)


def test_illumination_checkpoints_resume_bitwise(fpm, tmp_path):
    # ReconstructionCheckpoint carries the corrections (src/reconstruction/
    # checkpoint.rs:44); a run split at checkpoints, and one resumed from a
    # saved file, reproduce the uninterrupted run bit for bit.
    model, omodel, data = _case(fpm, 3, 32, seed=66)
    problem = fpm.ReconstructionProblem(data, model)
    algo = fpm.GradientDescent(iterations=6, recover_illumination=True, illumination_step=0.5)
    straight = algo.run(problem)
    staged = algo.run(problem, callbacks=[fpm.CheckpointEvery(2, tmp_path)])
    np.testing.assert_array_equal(straight.object_spectrum, staged.object_spectrum)
    np.testing.assert_array_equal(straight.calibrated_illumination, staged.calibrated_illumination)
    cp = fpm.ReconstructionCheckpoint.load(tmp_path / "checkpoint_00004.json")
    assert cp.illumination_corrections.shape == (model.frame_count, 2)
    assert np.abs(cp.illumination_corrections).max() > 0.0
    resumed = algo.run(problem, resume_from=cp)
    np.testing.assert_array_equal(straight.object_spectrum, resumed.object_spectrum)
    np.testing.assert_array_equal(straight.calibrated_illumination, resumed.calibrated_illumination)
    np.testing.assert_array_equal([t[1] for t in straight.trace], [t[1] for t in resumed.trace])
