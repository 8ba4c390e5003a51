"""Pose covariances (set_compute_covariances) against the inverse of the
Gauss-Newton matrix J^T J built in numpy from the FP64 evaluator's Jacobians
at the final state, with the GPS prior terms: the covariance Ceres computes
for BundleAdjuster::ComputeCovariances (bundle_adjuster.cc:1217-1287).

Bars: FP64 solve 1e-8 relative (of the block's largest entry), mixed 1e-4
(FP32 records)."""
import dataclasses

import numpy as np
import pytest

from opensfm_gb300 import _lib
from opensfm_gb300 import synthetic as syn
from opensfm_gb300.pybundle import adjuster_from_scene
from opensfm_gb300.scene import evaluate_projections

pytestmark = pytest.mark.gpu


def _reference_covariances(scene, ba):
    ni = len(scene.rig_instance_poses)
    poses = np.array([ba.get_rig_instance_pose(str(i)).ba_data() for i in range(ni)])
    final = dataclasses.replace(scene, rig_instance_poses=poses, points=ba.get_points())
    ev = evaluate_projections(final, _lib.PRECISION_FP64)
    npt = len(final.points)
    n = 6 * ni + 3 * npt
    H = np.zeros((n, n))
    inst = final.shot_rig_instance[final.obs_shot]
    for o in range(final.n_observations):
        cols = np.r_[6 * inst[o] + np.arange(6), 6 * ni + 3 * final.obs_point[o] + np.arange(3)]
        J = np.hstack([ev.jac_instance[o], ev.jac_point[o]])
        H[np.ix_(cols, cols)] += J.T @ J
    # GPS priors on the camera centres: r = (c - gps) / sigma
    for s in range(len(final.shot_camera)):
        i = int(final.shot_rig_instance[s])
        for k in range(3):
            H[6 * i + 3 + k, 6 * i + 3 + k] += 1.0 / scene.extras["gps_std"][s][k] ** 2
    C = np.linalg.inv(H)
    return [C[6 * i:6 * i + 6, 6 * i:6 * i + 6] for i in range(ni)]


@pytest.mark.parametrize("precision,bar", [("fp64", 1e-8), ("mixed", 1e-4)])
@pytest.mark.parametrize("solver", ["DENSE_SCHUR", "ITERATIVE_SCHUR"])
def test_pose_covariances_match_inverse_gauss_newton(precision, bar, solver):
    scene = syn.aerial_scene(seed=3, nx=4, ny=4, n_points=300)
    ba = adjuster_from_scene(scene, precision=precision, loss=None, irls="none", gps=True, constant_cameras=True,
                             max_iterations=50, linear_solver=solver, covariances=True,
                             pcg_tolerance=1e-10 if precision == "fp64" else 1e-4)
    ba.run()
    assert ba.get_covariance_estimation_valid()
    ref = _reference_covariances(scene, ba)
    for i, r in enumerate(ref):
        got = ba.get_rig_instance_covariance(str(i))
        np.testing.assert_allclose(got, got.T, atol=1e-12 * np.abs(got).max())
        assert np.abs(got - r).max() <= bar * np.abs(r).max(), (i, np.abs(got - r).max(), np.abs(r).max())


def test_gauge_free_problem_gives_the_default():
    # no priors: J^T J is singular (similarity gauge); the reference's
    # fallback covariance is stored and the estimate is flagged invalid
    scene = syn.ring_scene(n_points=300)
    ba = adjuster_from_scene(scene, precision="fp64", loss=None, irls="none", gps=False, constant_cameras=True,
                             max_iterations=20, covariances=True)
    ba.run()
    assert not ba.get_covariance_estimation_valid()
    c = ba.get_rig_instance_covariance("0")
    np.testing.assert_array_equal(np.diag(c), [1e-5] * 3 + [1e-2] * 3)
