"""BundleFull / BundleLocalStochastic helpers on the host (no GPU): control
point triangulation, the bias-parameter and alignment choices, the control
point set-up and the write-back checks (ba_helpers.cc:442-936, 1372-1845).
"""
import types

import numpy as np
import pytest

from opensfm_gb300 import ba_helpers as bh
from opensfm_gb300 import pybundle
from opensfm_gb300 import synthetic as syn
from opensfm_gb300.pygeometry import Pose, Similarity


def small_aerial(seed=3, **kw):
    scene = syn.aerial_scene(seed=seed, nx=6, ny=6, n_points=1500, offset=(0.0, 0.0, 0.0), **kw)
    return scene


def control_points(scene, idx, noise=0.0, seed=0, use_true_obs=True):
    """Control points at scene points `idx`: their observations projected
    from the true poses (noise-free unless `noise`), their true positions."""
    rng = np.random.default_rng(seed)
    true_xy = syn.project_scene(scene, scene.extras["true_poses"], scene.extras["true_points"])
    gcps = []
    for k, p in enumerate(idx):
        obs = np.nonzero(np.asarray(scene.obs_point) == p)[0]
        ob = [(int(scene.obs_shot[o]), true_xy[o] + rng.normal(0, noise, 2)) for o in obs]
        gcps.append(bh.GroundControlPoint(id=str(k), observations=ob, position=scene.extras["true_points"][p].copy()))
    return gcps


def at_truth(scene):
    scene.rig_instance_poses = scene.extras["true_poses"].copy()
    scene.points = scene.extras["true_points"].copy()
    return scene


def test_triangulate_gcp_exact_and_rejects_an_outlier_ray():
    scene = at_truth(small_aerial())
    counts = np.bincount(np.asarray(scene.obs_point))
    p = int(np.argmax(counts))
    g = control_points(scene, [p])[0]
    ok, X, inl = bh.triangulate_gcp(g, scene, threshold=0.05)
    assert ok and inl.all()
    np.testing.assert_allclose(X, scene.extras["true_points"][p], atol=1e-6)
    # one observation far off: outside the angular threshold, not an inlier
    g.observations[0] = (g.observations[0][0], g.observations[0][1] + 0.2)
    ok, X, inl = bh.triangulate_gcp(g, scene, threshold=0.05)
    assert ok and not inl[0] and inl[1:].all()
    np.testing.assert_allclose(X, scene.extras["true_points"][p], atol=1e-6)
    # fewer than two rays, or unknown shots only
    assert not bh.triangulate_gcp(bh.GroundControlPoint("x", g.observations[:1]), scene, 0.05)[0]
    assert not bh.triangulate_gcp(bh.GroundControlPoint("x", [(10_000, np.zeros(2))] * 3), scene, 0.05)[0]


def test_gcp_bias_parameters_follow_the_control_point_layout():
    scene = at_truth(small_aerial())
    counts = np.bincount(np.asarray(scene.obs_point))
    good = np.nonzero(counts >= 3)[0]
    X = scene.extras["true_points"]
    assert bh.determine_gcp_bias_parameters(scene, [], {}) == list(range(7))
    assert bh.determine_gcp_bias_parameters(scene, control_points(scene, good[:1]), {}) == [3, 4, 5]
    assert bh.determine_gcp_bias_parameters(scene, control_points(scene, good[:2]), {}) == [3, 4, 5, 6]
    # three spread points: all parameters
    far = [good[0], good[np.argmax(np.linalg.norm(X[good] - X[good[0]], axis=1))]]
    d = np.abs(np.cross(X[good] - X[far[0]], X[far[1]] - X[far[0]])).sum(axis=1)
    third = good[np.argmax(d)]
    assert bh.determine_gcp_bias_parameters(scene, control_points(scene, far + [third]), {}) == list(range(7))


def test_collinearity_and_alignment_detection():
    line = np.array([[0, 0, 0], [1, 1, 1], [2, 2, 2], [3, 3, 3.0]])
    assert bh.are_points_collinear(line)
    assert not bh.are_points_collinear(np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1.0]]))
    scene = small_aerial()
    assert bh.detect_alignment_constraints(scene, [], {}) == "naive"          # GPS on a 6 x 6 grid
    assert bh.detect_alignment_constraints(scene, [], {"bundle_use_gps": False}) == "orientation_prior"
    assert bh._up_vector(scene, [], bh._config({"align_method": "orientation_prior"}))[1] == -1.0
    assert bh.determine_linear_solver(200) == "DENSE_SCHUR" and bh.determine_linear_solver(201) == "SPARSE_SCHUR"


def test_add_gcp_to_bundle_adds_points_and_observations():
    scene = at_truth(small_aerial())
    counts = np.bincount(np.asarray(scene.obs_point))
    good = np.nonzero(counts >= 3)[0][:3]
    gcps = control_points(scene, good)
    gcps.append(bh.GroundControlPoint("check", gcps[0].observations, gcps[0].position, role="checkpoint"))
    ba = pybundle.BundleAdjuster()
    from opensfm_gb300.pygeometry import Camera
    cam = Camera(int(scene.camera_projection[0]), scene.camera_values[0, :3])
    ba.add_camera("0", cam, cam, True)
    ba.add_rig_camera("rig", Pose(), Pose(), True)
    for s in range(len(scene.shot_camera)):
        ba.add_rig_instance(str(s), Pose.from_ba_data(scene.rig_instance_poses[s]), {str(s): "0"}, {str(s): "rig"},
                            False)
    added = bh.add_gcp_to_bundle(ba, scene, gcps, {}, 1000, 36, set(range(36)))
    assert added == sum(len(g.observations) for g in gcps[:3])
    for k in range(3):
        assert ba.has_point(f"gcp-{k}")
    assert not ba.has_point("gcp-check")


class _FakeAdjuster:
    def __init__(self, n_inst, pts, bad_pose=None):
        self.n_inst, self.pts, self.bad_pose = n_inst, pts, bad_pose

    def get_camera(self, k):
        raise AssertionError("cameras are not updated")

    def get_bias(self, k):
        return Similarity()

    def get_rig_instance_pose(self, i):
        d = np.zeros(6)
        if self.bad_pose == int(i):
            d[0] = np.nan
        return types.SimpleNamespace(ba_data=lambda: d)

    def get_points(self):
        return self.pts

    def projection_results(self):
        n = self.n
        return np.zeros((n, 3)), np.ones(n), np.full(n, 2)


def test_bundle_to_map_refuses_non_finite_poses_and_flags_non_finite_points():
    scene = small_aerial()
    pts = np.array(scene.points, copy=True)
    pts[3] = np.nan
    fake = _FakeAdjuster(len(scene.rig_instance_poses), pts, bad_pose=2)
    fake.n = scene.n_observations
    with pytest.raises(RuntimeError, match="Rig Instance 2 has either NaN or INF values."):
        bh.bundle_to_map(fake, scene, update_cameras=False)
    fake.bad_pose = None
    out = bh.bundle_to_map(fake, scene, update_cameras=False)
    bad = np.asarray(scene.obs_point) == 3
    assert np.all(out["errors"][bad] == 1.0) and np.all(out["weights"][bad] == 0.0)
    assert np.all(out["weights"][~bad] == 1.0)
    assert np.isnan(scene.points[3]).all()


def test_gps_accuracy_must_be_positive():
    scene = small_aerial()
    scene.extras["gps_std"] = np.array(scene.extras["gps_std"], copy=True)
    scene.extras["gps_std"][4, 1] = 0.0
    with pytest.raises(RuntimeError, match="Shot 4 has an accuracy component <= 0"):
        bh._instance_gps(scene, [4])
