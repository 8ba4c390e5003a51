"""Adjusted GPS standard deviations (no GPU): the prior residual divided by a
per-scale-group std multiplier and the StdDeviationConstraint regulariser on
that multiplier (bundle_adjuster.cc:1049-1085, prior_error.h:54-93,
parameters_errors.h:7-16).  The library's host terms are checked against the
oracle's restatement and closed forms; the oracle's solve with these terms
is checked for stationarity in the multiplier.  The GPU solve against the
oracle is in test_gpu_position_std.py."""
import numpy as np
import pytest
from scipy.optimize import brentq

from oracle import oracle
from opensfm_gb300 import pybundle
from opensfm_gb300 import synthetic as syn

C = 0.5 * np.log(2 * np.pi)


@pytest.mark.parametrize("m", [0.3, 1.0, 2.7])
def test_gps_std_residual_matches_oracle(m):
    rng = np.random.default_rng(3)
    pose = np.r_[rng.normal(0, 0.4, 3), rng.normal(0, 5, 3)]
    prior, std = rng.normal(0, 5, 3), rng.uniform(0.1, 2.0, 3)
    r, J = pybundle.relative_residual("gps_std", pose[None], np.r_[prior, std, m])
    ro, Jo = oracle.relative_residual("gps_std", pose[None], np.r_[prior, std, 0.0], scales=[m, 1.0])
    np.testing.assert_allclose(r, (pose[3:] - prior) / (std * m), rtol=1e-14)
    np.testing.assert_allclose(r, ro, rtol=1e-14)
    np.testing.assert_allclose(J, Jo, rtol=1e-13, atol=1e-15)
    # position columns 3-5, the multiplier column 24, nothing else
    np.testing.assert_allclose(J[:, 3:6], np.diag(1 / (std * m)), rtol=1e-14)
    np.testing.assert_allclose(J[:, 24], -r / m, rtol=1e-14)
    rest = np.delete(J, [3, 4, 5, 24], axis=1)
    assert not rest.any()


@pytest.mark.parametrize("m", [0.05, 1 / np.sqrt(2 * np.pi), 4.0])
def test_std_deviation_residual(m):
    r, J = pybundle.relative_residual("std_deviation", None, [m])
    ro, Jo = oracle.relative_residual("std_deviation", np.zeros((1, 6)), [0.0], scales=[m, 1.0])
    np.testing.assert_allclose(r, [-(np.log(m) + C)], rtol=1e-14, atol=1e-15)
    np.testing.assert_allclose(r, ro, rtol=1e-14, atol=1e-15)
    np.testing.assert_allclose(J[0, 24], -1 / m, rtol=1e-14)
    np.testing.assert_allclose(J, Jo, rtol=1e-14)
    assert not np.delete(J, 24, axis=1).any()


def _adjusted_terms(scene):
    """The relative-term form of adjusted GPS priors: one multiplier
    (scale 0) shared by every shot's prior, plus its regulariser."""
    gps, std = scene.extras["gps"], scene.extras["gps_std"]
    rel = [("gps_std", (s,), np.r_[gps[s], std[s], 0.0]) for s in range(len(gps))]
    return rel + [("std_deviation", (), [0.0])]


def test_oracle_multiplier_is_optimal():
    # f(m) = A / (2 m^2) + (log m + c)^2 / 2 with A the sum of the squared
    # std-normalised GPS errors at the solution; f'(m*) = 0 <=>
    # (log m* + c) m*^2 = A.  The solve stops on Ceres' function tolerance
    # (relative cost change 1e-6), so the multiplier's part of the cost is
    # within that of its optimum, not m of m*
    scene = syn.ring_scene(n_points=300, seed=5)
    true = scene.extras["true_poses"]
    n = len(scene.shot_camera)
    rng = np.random.default_rng(8)
    scene.extras["gps"] = np.ascontiguousarray(true[:, 3:] + rng.normal(0, 0.3, (n, 3)))
    scene.extras["gps_std"] = np.full((n, 3), 0.1)
    ref = oracle.solve(scene, loss=("HuberLoss", 1.0), irls="none", max_iterations=200, gps=False,
                       relative=_adjusted_terms(scene), scales=[(1.0, True)])
    assert ref["termination"] == 1
    m = ref["scales"][0]
    pos = ref["instances"][scene.shot_rig_instance][:, 3:]
    A = np.sum(((pos - scene.extras["gps"]) / scene.extras["gps_std"]) ** 2)
    assert m > 1.0  # GPS noise three times its stated std
    m_star = brentq(lambda x: (np.log(x) + C) * x * x - A, 1e-3, 1e3)

    def f(x):
        return A / (2 * x * x) + (np.log(x) + C) ** 2 / 2

    assert 0 <= f(m) - f(m_star) < 1e-6 * ref["final_cost"]
    np.testing.assert_allclose(m, m_star, rtol=1e-2)


def test_batch_set_up_drops_the_multiplier_and_restores_the_priors():
    # a batch rejects the multiplier (a free camera-side block) on the host,
    # before any device work; the failed set-up leaves the adjuster as it
    # was, so the next set-up without adjusting meets the GPS priors again
    scene = syn.ring_scene(n_points=100, seed=5)
    n = len(scene.shot_camera)
    scene.extras["gps"] = np.ascontiguousarray(scene.extras["true_poses"][:, 3:])
    scene.extras["gps_std"] = np.full((n, 3), 0.1)
    ba = pybundle.adjuster_from_scene(scene, precision="mixed", irls="none", constant_cameras=True)
    ba.set_adjust_absolute_position_std(True)
    batch = pybundle.BundleBatch()
    batch.add(ba)
    with pytest.raises(Exception, match="fixed rig cameras"):
        batch.run()
    with pytest.raises(Exception, match="fixed rig cameras"):
        batch.run()
    ba.set_adjust_absolute_position_std(False)
    with pytest.raises(Exception, match="no position priors"):
        batch.run()
