"""The single-CTA frame engine for 256-point tiles (fpm_set_engine_shape).

Both engine shapes compute every value with the same arithmetic in the same
order, so their objects agree to the last bits; each is also checked against
the FP64 oracle (complex NRMSE <= 1e-4, objectives to 1e-4 relative). Cases:
AP, FPIE, mPIE and EPRY without pupil recovery; a unit pupil (read from its
row spans) and an aberrated one (read from memory); masked amplitude-form
measurements; a non-sequential schedule; fewer CTAs than tiles.
"""

from __future__ import annotations

import numpy as np
import pytest

import helpers
import oracle
import workloads as W

pytestmark = pytest.mark.gpu

NRMSE = 1e-4
# The two engine shapes: same per-value arithmetic, so the difference is at
# most FP32 contraction noise.
ENGINES_AGREE = 1e-6


@pytest.fixture(scope="module")
def fpm(native_library):
    import fpm_rs

    yield fpm_rs
    fpm_rs.tuning.apply({}, {256: fpm_rs.tuning.AUTO})


def _both_shapes(fpm, algo, problems, schedule="sequential"):
    fpm.tuning.apply({}, {256: fpm.tuning.CLUSTER})
    cluster = fpm.run_batch(algo, problems, schedule=schedule)
    fpm.tuning.apply({}, {256: fpm.tuning.SINGLE_CTA})
    single = fpm.run_batch(algo, problems, schedule=schedule)
    assert fpm.last_run_stats()["engine_launches"] >= 1
    return cluster, single


def _objective_close(gpu, cpu, rtol=1e-4):
    gpu, cpu = np.asarray(gpu), np.asarray(cpu)
    assert np.all(np.abs(gpu - cpu) <= rtol * np.abs(cpu) + 1e-12), (gpu, cpu)


ALGOS = {
    "ap": (lambda fpm: fpm.AlternatingProjection(iterations=3), dict(iterations=3)),
    "fpie": (lambda fpm: fpm.Fpie(iterations=3), dict(iterations=3)),
    "mpie": (lambda fpm: fpm.Mpie(iterations=3, momentum_interval=7), dict(iterations=3, momentum_interval=7)),
    "epry": (lambda fpm: fpm.Epry(iterations=3, recover_pupil=False), dict(iterations=3, recover_pupil=False)),
}


@pytest.mark.parametrize("alg", sorted(ALGOS))
def test_single_cta_engine_matches_cluster_and_oracle(fpm, alg):
    make, kw = ALGOS[alg]
    model, omodel, data, truth, gains = helpers.simulated(fpm, 5, 256, seed=31, photons=1e4)
    problem = fpm.ReconstructionProblem(data, model)
    cluster, single = _both_shapes(fpm, make(fpm), [problem])
    assert oracle.complex_nrmse(cluster[0].object, single[0].object) <= ENGINES_AGREE
    expected = oracle.run(oracle.Problem(omodel, data, gains=gains), alg, **kw)
    assert oracle.complex_nrmse(expected["object"], single[0].object) <= NRMSE
    _objective_close([t[1] for t in single[0].trace], expected["objectives"])


def test_aberrated_pupil_masks_and_schedule(fpm):
    """A complex (non-unit) pupil is read from memory; masked pixels in the
    amplitude form; the spiral-out frame order."""
    model, omodel, data, truth, gains = helpers.simulated(fpm, 5, 256, seed=32, photons=1e4)
    pupil = W.zernike_pupil(omodel["support"], 12)
    model = model._replace(pupil=pupil)
    omodel = dict(omodel, pupil=pupil)
    masks = (np.random.default_rng(4).random(data.shape) > 0.1).astype(np.uint8)
    problem = fpm.ReconstructionProblem(data, model, masks=masks)
    algo = fpm.Mpie(iterations=2, momentum_interval=9)
    cluster, single = _both_shapes(fpm, algo, [problem], schedule="spiral_out")
    assert oracle.complex_nrmse(cluster[0].object, single[0].object) <= ENGINES_AGREE
    expected = oracle.run(oracle.Problem(omodel, data, gains=gains, masks=masks), "mpie", iterations=2,
                          momentum_interval=9, schedule="spiral_out")
    assert oracle.complex_nrmse(expected["object"], single[0].object) <= NRMSE
    _objective_close([t[1] for t in single[0].trace], expected["objectives"])


def test_fewer_ctas_than_tiles_give_the_same_bits(fpm):
    problems = []
    for k in range(5):
        model, omodel, data, truth, gains = helpers.simulated(fpm, 3, 256, seed=40 + k, photons=1e4)
        problems.append(fpm.ReconstructionProblem(data, model))
    algo = fpm.Mpie(iterations=2, momentum_interval=5)
    fpm.tuning.apply({}, {256: fpm.tuning.SINGLE_CTA})
    expected = fpm.run_batch(algo, problems)
    fpm.tuning.apply({}, {256: fpm.tuning.SINGLE_CTA}, {256: 2})
    got = fpm.run_batch(algo, problems)
    fpm.tuning.apply({}, {256: fpm.tuning.SINGLE_CTA}, {256: 0})
    for a, b in zip(expected, got):
        assert np.array_equal(a.object, b.object)
        assert [t[1] for t in a.trace] == [t[1] for t in b.trace]


def test_auto_shape_takes_the_cluster_engine_for_few_tiles(fpm):
    """AUTO (the default for 256) gives a lone tile the cluster engine: the
    result equals the explicit cluster shape's to the bit."""
    model, omodel, data, truth, gains = helpers.simulated(fpm, 3, 256, seed=50, photons=1e4)
    problem = fpm.ReconstructionProblem(data, model)
    algo = fpm.Mpie(iterations=1)
    fpm.tuning.apply({}, {256: fpm.tuning.CLUSTER})
    cluster = fpm.run_batch(algo, [problem])
    fpm.tuning.apply({}, {256: fpm.tuning.AUTO})
    auto = fpm.run_batch(algo, [problem])
    assert np.array_equal(cluster[0].object, auto[0].object)
    assert [t[1] for t in cluster[0].trace] == [t[1] for t in auto[0].trace]


def test_engine_shape_validation(fpm):
    from fpm_rs.errors import FpmError

    with pytest.raises(FpmError):
        fpm.tuning.set_engine_shape(128, fpm.tuning.SINGLE_CTA)
    with pytest.raises(FpmError):
        fpm.tuning.set_engine_shape(256, 7)
    assert fpm.tuning.max_clusters(256) >= 1
