"""The oracle's non-projection terms pinned to the reference's own expected
values (no GPU): opensfm/test/test_bundle.py's singleton, relative-motion
and heatmap cases, solved by the oracle's FP64 LM on scenes with no
observations.  The GPU solves of the same cases are in
test_gpu_orientation.py, test_gpu_relative.py and
test_gpu_relative_motion.py."""
import numpy as np
import pytest

from oracle import oracle
from opensfm_gb300 import pygeometry
from opensfm_gb300 import scene as sc


def _scene(poses, gps=None):
    """Shots 0..n-1, one per rig instance, a fixed unit-focal camera, no
    points; ``gps``: per shot (position, std) or None."""
    n = len(poses)
    s = sc.SceneArrays(
        camera_projection=[sc.PERSPECTIVE], camera_values=np.array([[0.0, 0.0, 1.0]]),
        rig_instance_poses=np.array([p.ba_data() for p in poses]), shot_rig_instance=np.arange(n),
        shot_camera=np.zeros(n), points=np.zeros((0, 3)), obs_shot=np.zeros(0, np.int32),
        obs_point=np.zeros(0, np.int32), obs_xy=np.zeros((0, 2)), obs_std=np.zeros(0))
    if gps is not None:
        s.extras["gps"] = np.array([g[0] for g in gps], np.float64)
        s.extras["gps_std"] = np.array([g[1] for g in gps], np.float64)
    return s


def _solve(scene, **kw):
    r = oracle.solve(scene, irls="none", max_iterations=100, gps="gps" in scene.extras, constant_cameras=True, **kw)
    assert r["termination"] == 1, r
    return r, [pygeometry.Pose.from_ba_data(p) for p in r["instances"]]


def _motion(i, j, t, si, sj, observed=False):
    return ("relative_motion", (i, j), np.r_[0, 0, 0, t, 1, float(observed), np.eye(7).ravel(), 1, si, sj])


@pytest.mark.parametrize("shared,expected", [(True, [0.5]), (False, [4.0, 0.5])])
def test_pair(shared, expected):
    # test_bundle.py:167-194 and :268-295
    s = _scene([pygeometry.Pose()] * 2, gps=[([0, 0, 0], [1, 1, 1]), ([2, 0, 0], [1, 1, 1])])
    r, poses = _solve(s, relative=[_motion(0, 1, [-1, 0, 0], 0, 0 if shared else 1)],
                      scales=[(4.0, True)] * (1 if shared else 2))
    np.testing.assert_allclose(poses[0].translation, [0, 0, 0], atol=1e-6)
    np.testing.assert_allclose(poses[1].translation, [-2, 0, 0], atol=1e-6)
    np.testing.assert_allclose(r["scales"], expected, atol=1e-6)


def test_four_cams_single_reconstruction():
    # test_bundle.py:298-362: one shared scale
    s = _scene([pygeometry.Pose()] * 4, gps=[([0, 0, 0], [1, 1, 1]), ([2, 0, 0], [1, 1, 1]),
                                             ([0, 2, 0], [1, 1, 1]), ([0, 0, 0], [1e9, 1e9, 1e9])])
    rel = [_motion(0, 1, [-1, 0, 0], 0, 0), _motion(0, 2, [0, -1, 0], 0, 0), _motion(0, 3, [0, 0, -1], 0, 0)]
    _, poses = _solve(s, relative=rel, scales=[(1.0, True)])
    for p, t in zip(poses, ([0, 0, 0], [-2, 0, 0], [0, -2, 0], [0, 0, -2])):
        np.testing.assert_allclose(p.translation, t, atol=1e-5)


def test_four_cams_double_reconstruction():
    # test_bundle.py:365-452: per-instance scales, two of the scales observed
    s = _scene([pygeometry.Pose()] * 4, gps=[([0, 0, 0], [1, 1, 1]), ([0, 0, 0], [1e9, 1e9, 1e9]),
                                             ([0, 0, 0], [1e9, 1e9, 1e9]), ([3, 3, 3], [1, 1, 1])])
    rel = [_motion(0, 1, [-0.5, -0.5, -0.5], 0, 1, observed=True), _motion(2, 1, [0.5, 0.5, 0.5], 2, 1),
           _motion(2, 3, [-2, -2, -2], 2, 3, observed=True), _motion(1, 2, [-2, -2, -2], 1, 2)]
    r, poses = _solve(s, relative=rel, scales=[(1.0, True)] * 4)
    for p, o in zip(poses, ([0, 0, 0], [1, 1, 1], [2, 2, 2], [3, 3, 3])):
        np.testing.assert_allclose(p.get_origin(), o, atol=1e-5)
    np.testing.assert_allclose(r["scales"], [0.5, 0.5, 2.0, 2.0], atol=1e-5)


def test_singleton_up_vector_and_pan():
    # test_bundle.py:47-65
    s = _scene([pygeometry.Pose(np.array([0.5, 0, 0]), np.zeros(3))], gps=[([1, 0, 0], [1, 1, 1])])
    _, poses = _solve(s, orientation=[("up_vector", 0, [0, -1, 0], 1.0), ("pan", 0, np.radians(180), 1.0)])
    np.testing.assert_allclose(poses[0].translation, [1, 0, 0], atol=1e-6)


def test_singleton_pan_tilt_roll():
    # test_bundle.py:68-92
    pan, tilt, roll = 1.0, 0.3, 0.2
    s = _scene([pygeometry.Pose(np.array([0.5, 0, 0]), np.zeros(3))], gps=[([1, 0, 0], [1, 1, 1])])
    _, poses = _solve(s, orientation=[("pan", 0, pan, 1.0), ("tilt", 0, tilt, 1.0), ("roll", 0, roll, 1.0)])
    np.testing.assert_allclose(poses[0].get_origin(), [1, 0, 0], atol=1e-6)
    R = poses[0].get_rotation_matrix()
    z, x = R.T @ [0, 0, 1], R.T @ [1, 0, 0]
    a = np.cross(z, [0, 0, 1])
    a /= np.linalg.norm(a)
    got = (np.arctan2(z[0], z[1]), np.arctan2(-z[2], np.linalg.norm(z[:2])), np.arcsin(np.dot(z, np.cross(x, a))))
    np.testing.assert_allclose(got, (pan, tilt, roll), atol=1e-6)


def test_heatmap_singletons():
    # test_bundle.py:650-735 (without its reconstruction bookkeeping)
    size, rad, hx, hy = 101, 10.0, 1.0, -1.0
    res = 2 * rad / (size - 1)
    x, y = np.meshgrid(np.linspace(-rad, rad, size), np.linspace(rad, -rad, size))
    z = np.exp(-((x - hx) ** 2 / (2 * (rad / 2) ** 2) + (y - hy) ** 2 / (2 * (rad / 2) ** 2)))
    grid = 1 - z / z.max()
    offsets = [(2, 0), (0, 2), (-2, 0)]
    s = _scene([pygeometry.Pose(np.full(3, 0.0), np.zeros(3))] * 3)
    rel = [("heatmap", (i,), [xo, yo, 1.0]) for i, (xo, yo) in enumerate(offsets)]
    _, poses = _solve(s, relative=rel, heatmap=(grid, size, res))
    for p, (xo, yo) in zip(poses, offsets):
        np.testing.assert_allclose(-p.translation, [xo + hx, yo + hy, 0], atol=res)


def test_four_cams_one_fixed():
    # test_bundle.py:455-526: the fixed instance ignores its own GPS prior
    s = _scene([pygeometry.Pose()] * 4, gps=[([100, 0, 0], [1, 1, 1]), ([2, 0, 0], [1, 1, 1]),
                                             ([0, 2, 0], [1, 1, 1]), ([0, 0, 0], [1e9, 1e9, 1e9])])
    rel = [_motion(0, 1, [-1, 0, 0], 0, 0), _motion(0, 2, [0, -1, 0], 0, 0), _motion(0, 3, [0, 0, -1], 0, 0)]
    _, poses = _solve(s, relative=rel, scales=[(1.0, True)], fixed_instances=[0])
    for p, t in zip(poses, ([0, 0, 0], [-2, 0, 0], [0, -2, 0], [0, 0, -2])):
        np.testing.assert_allclose(p.translation, t, atol=1e-6)


def test_linear_motion_prior_position():
    # test_bundle.py:529-552: the middle instance has no GPS
    s = _scene([pygeometry.Pose()] * 3, gps=[([0, 0, 0], [1, 1, 1]), ([0, 0, 0], [1e9, 1e9, 1e9]),
                                             ([2, 0, 0], [1, 1, 1])])
    _, poses = _solve(s, relative=[("linear_motion", (0, 1, 2), [0.5, 0.1, 0.1])])
    for p, t in zip(poses, ([0, 0, 0], [-1, 0, 0], [-2, 0, 0])):
        np.testing.assert_allclose(p.translation, t, atol=1e-6)


def test_linear_motion_prior_rotation():
    # test_bundle.py:555-590: the end instances held, the middle rotation
    # interpolated at alpha = 0.3
    s = _scene([pygeometry.Pose(), pygeometry.Pose(), pygeometry.Pose(np.array([0, 1.0, 0]), np.zeros(3))])
    _, poses = _solve(s, relative=[("linear_motion", (0, 1, 2), [0.3, 0.1, 0.1])], fixed_instances=[0, 2])
    np.testing.assert_allclose(poses[1].rotation, [0, 0.3, 0], atol=1e-6)
