"""BundleFull and BundleLocalStochastic on the GPU adjuster
(ba_helpers.cc:442-804, 1372-1671): a small aerial scene whose GPS carries
a known similarity bias, with ground control points that fix the frame.
The full bundle with GPS-bias compensation recovers the bias and the camera
centres; a stochastic local bundle moves only its interior instances and
carries the bias on from the scene.
"""
import numpy as np
import pytest

from opensfm_gb300 import ba_helpers as bh
from opensfm_gb300 import synthetic as syn
from test_ba_full_host import control_points

pytestmark = pytest.mark.gpu

BIAS = (np.array([0.004, -0.006, 0.005]), np.array([3.0, -2.0, 1.5]), 1.01)


def biased_scene(seed=3):
    scene = syn.aerial_scene(seed=seed, nx=8, ny=8, n_points=3000, offset=(0.0, 0.0, 0.0), gps_sigma=(0.2, 0.2, 0.4))
    w, t, s = BIAS
    scene.extras["gps"] = ((scene.extras["gps"] - t) / s) @ syn.rotation_matrix(w)
    X = scene.extras["true_points"]
    counts = np.bincount(np.asarray(scene.obs_point))
    good = np.nonzero(counts >= 4)[0]
    # four control points near the corners of the block
    lo, hi = X[good].min(axis=0), X[good].max(axis=0)
    corners = [(lo[0], lo[1]), (lo[0], hi[1]), (hi[0], lo[1]), (hi[0], hi[1])]
    idx = [int(good[np.argmin(np.hypot(X[good, 0] - cx, X[good, 1] - cy))]) for cx, cy in corners]
    gcps = control_points(scene, idx, noise=1e-4, seed=seed)
    return scene, gcps


CONFIG = {"bundle_compensate_gps_bias": True, "optimize_camera_parameters": False, "bundle_max_iterations": 60}


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_bundle_full_compensates_the_gps_bias(precision):
    scene, gcps = biased_scene()
    d0 = np.linalg.norm(scene.rig_instance_poses[:, 3:] - scene.extras["true_poses"][:, 3:], axis=1)
    rep = bh.bundle_full(scene, CONFIG, gcps, grid_size=1, precision=precision)
    assert rep["is_solution_usable"]
    assert rep["summary"]["final_cost"] < rep["summary"]["initial_cost"]
    assert rep["num_points"] == len(scene.points) and rep["num_images"] == 64
    b = scene.extras["biases"]["0"]
    w, t, s = BIAS
    assert np.abs(b.rotation - w).max() < 2e-3
    assert np.abs(b.translation - t).max() < 0.3
    assert abs(b.scale - s) < 2e-3
    # the control points fix the frame (their priors weigh gcp_vertical_sd
    # 0.1 m / (0.04 sqrt(points per shot)) ~ 0.37 m vertically): the camera
    # centres move to within a fraction of their initial error of the truth
    d = np.linalg.norm(scene.rig_instance_poses[:, 3:] - scene.extras["true_poses"][:, 3:], axis=1)
    assert np.median(d) < 0.5 * np.median(d0), (np.median(d), np.median(d0))
    assert np.all(np.isfinite(rep["reprojection"]["errors"]))


def test_bundle_full_without_bias_keeps_it_and_updates_cameras():
    scene, gcps = biased_scene(seed=5)
    cam0 = scene.camera_values.copy()
    rep = bh.bundle_full(scene, {"bundle_max_iterations": 30}, gcps, grid_size=1, precision="fp64")
    assert rep["is_solution_usable"]
    assert not np.array_equal(scene.camera_values, cam0)        # optimize_camera_parameters is on by default
    b = scene.extras["biases"]["0"]
    np.testing.assert_array_equal(b.translation, np.zeros(3))   # compensation off: the bias is not a parameter


def test_bundle_local_stochastic_moves_the_interior_only():
    scene, gcps = biased_scene(seed=7)
    before = scene.rig_instance_poses.copy()
    pts_before = scene.points.copy()
    cfg = dict(CONFIG, local_bundle_max_shots=12, local_bundle_radius=3, local_bundle_min_common_points=20,
               bundle_max_iterations=20)
    ids, rep = bh.bundle_local_stochastic(scene, [27], cfg, gcps, grid_size=1, precision="fp64")
    assert rep["is_solution_usable"]
    assert rep["num_interior_images"] <= 12
    moved = np.nonzero(np.any(scene.rig_instance_poses != before, axis=1))[0]
    assert len(moved) > 0 and len(moved) <= rep["num_interior_images"]
    untouched = np.setdiff1d(np.arange(64), moved)
    np.testing.assert_array_equal(scene.rig_instance_poses[untouched], before[untouched])
    assert not np.array_equal(scene.points[ids], pts_before[ids])
    others = np.setdiff1d(np.arange(len(scene.points)), ids)
    np.testing.assert_array_equal(scene.points[others], pts_before[others])
    # the bias moved from the identity toward the GPS bias
    assert np.linalg.norm(scene.extras["biases"]["0"].translation) > 0.5
