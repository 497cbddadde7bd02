"""Persistent frame-engine launches: with fewer clusters than tiles
(fpm_set_engine_grid) each cluster walks several tiles, and every tile's
result is bit-identical to the one-cluster-per-tile launch."""

from __future__ import annotations

import numpy as np
import pytest

import helpers

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def fpm(native_library):
    import fpm_rs

    yield fpm_rs
    fpm_rs.tuning.apply({})  # one cluster per tile again


def _problems(fpm, specs):
    out = []
    for side, n, seed in specs:
        model, omodel, data, truth, gains = helpers.simulated(fpm, side, n, seed=seed, photons=1e4)
        out.append(fpm.ReconstructionProblem(data, model))
    return out


@pytest.mark.parametrize("make", [
    lambda fpm: fpm.Mpie(iterations=3, momentum_interval=7),
    lambda fpm: fpm.GradientDescent(iterations=2, batch_size=4, object_tv=1e-3),
], ids=["mpie", "gd_tv"])
def test_fewer_clusters_than_tiles_give_the_same_bits(fpm, make):
    specs = [(3, 32, 60 + k) for k in range(5)] + [(5, 64, 70 + k) for k in range(4)] + \
            [(5, 128, 80 + k) for k in range(3)] + [(3, 256, 90 + k) for k in range(3)]
    problems = _problems(fpm, specs)
    algo = make(fpm)
    fpm.tuning.apply({})
    expected = fpm.run_batch(algo, problems)
    fpm.tuning.apply({"32": 2, "64": 3, "128": 1, "256": 2})
    got = fpm.run_batch(algo, problems)
    fpm.tuning.apply({})
    for a, b in zip(expected, got):
        assert np.array_equal(a.object, b.object)
        assert np.array_equal(a.recovered_pupil, b.recovered_pupil)
        assert [t[1] for t in a.trace] == [t[1] for t in b.trace]


def test_residency_limits(fpm):
    for n in (32, 64, 128, 256):
        assert fpm.tuning.max_clusters(n) >= 1
