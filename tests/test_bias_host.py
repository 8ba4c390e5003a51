"""Optimised camera biases (host side, no GPU).

SetCameraBias with parameters_to_optimize (bundle_adjuster.cc:131-140)
makes the bias -- geometry::Similarity, rotation RX RY RZ, translation TX TY
TZ, scale (bundle/data/bias.h:12) -- unknowns of every GPS prior whose
instance references the camera: DataPriorError with SimilarityPriorTransform
(prior_error.h:19-114, bias.h:34-54), residual (t - (s R(w) p + b)) / std
on the instance position t.  The library's host term is checked against the
oracle's restatement and central differences; the oracle's solve recovers a
known bias of the GPS; the getters round-trip.  The GPU solve against the
oracle is in test_gpu_bias.py.
"""
import numpy as np
import pytest

from oracle import oracle
from opensfm_gb300 import pybundle, pygeometry
from opensfm_gb300 import synthetic as syn


def _term(pose, prior, std, m, bias):
    w, b, s = bias[:3], bias[3:6], bias[6]
    pred = s * (syn.rotation_matrix(w) @ prior) + b
    return (pose[3:] - pred) / (std * m)


@pytest.mark.parametrize("m", [1.0, 0.7])
def test_gps_bias_residual_matches_oracle_and_differences(m):
    rng = np.random.default_rng(5)
    pose = np.r_[rng.normal(0, 0.4, 3), rng.normal(0, 5, 3)]
    prior, std = rng.normal(0, 5, 3), rng.uniform(0.1, 2.0, 3)
    bias = np.r_[rng.normal(0, 0.1, 3), rng.normal(0, 1, 3), 1.0 + 0.05 * rng.normal()]
    r, J = pybundle.relative_residual("gps_bias", pose[None], np.r_[prior, std, m, bias])
    np.testing.assert_allclose(r, _term(pose, prior, std, m, bias), rtol=1e-13)
    # the oracle: multiplier in column 24, bias in columns 12..18
    ro, Jo = oracle.relative_residual("gps_bias", pose[None], np.r_[prior, std, 0.0, np.arange(1, 8)],
                                      scales=np.r_[m, bias])
    np.testing.assert_allclose(r, ro, rtol=1e-13)
    np.testing.assert_allclose(J[:, 3:6], Jo[:, 3:6], rtol=1e-13)
    np.testing.assert_allclose(J[:, 6:12], Jo[:, 12:18], rtol=1e-12, atol=1e-14)
    np.testing.assert_allclose(J[:, 25], Jo[:, 18], rtol=1e-12)
    np.testing.assert_allclose(J[:, 24], Jo[:, 24], rtol=1e-12)
    # central differences of the closed form
    h = 1e-6
    for k in range(7):
        a, b = bias.copy(), bias.copy()
        a[k] += h
        b[k] -= h
        fd = (_term(pose, prior, std, m, a) - _term(pose, prior, std, m, b)) / (2 * h)
        col = 6 + k if k < 6 else 25
        np.testing.assert_allclose(J[:, col], fd, rtol=1e-6, atol=1e-8)
    rest = np.delete(J, [3, 4, 5, 6, 7, 8, 9, 10, 11, 24, 25], axis=1)
    assert not rest.any()


def test_gps_bias_residual_at_zero_rotation():
    # the bias starts at the identity: the first-order branch of the
    # rotation must still give the derivative -s [p]x / std
    pose = np.r_[0.1, 0.2, 0.3, 1.0, 2.0, 3.0]
    prior, std = np.array([4.0, -1.0, 2.0]), np.ones(3)
    bias = np.r_[0, 0, 0, 0, 0, 0, 1.0]
    _, J = pybundle.relative_residual("gps_bias", pose[None], np.r_[prior, std, 1.0, bias])
    px = np.array([[0, -prior[2], prior[1]], [prior[2], 0, -prior[0]], [-prior[1], prior[0], 0]])
    np.testing.assert_allclose(J[:, 6:9], px, atol=1e-15)  # d(-R(w)p)/dw at w = 0 is [p]x


def test_bias_setters_round_trip():
    ba = pybundle.BundleAdjuster()
    cam = pygeometry.Camera.create_perspective(1.0, 0.0, 0.0)
    ba.add_camera("c", cam, cam, True)
    b = pygeometry.Similarity([0.1, 0.0, -0.2], [1.0, 2.0, 3.0], 1.5)
    ba.set_camera_bias("c", b, [3, 4, 5, 6])
    got = ba.get_bias("c")
    np.testing.assert_array_equal(got.rotation, b.rotation)
    np.testing.assert_array_equal(got.translation, b.translation)
    assert got.scale == 1.5
    with pytest.raises(RuntimeError):
        ba.set_camera_bias("nope", b)
    with pytest.raises(RuntimeError):
        ba.set_camera_bias("c", b, [7])


def biased_aerial(seed=3):
    """A small aerial problem whose GPS carries a known similarity bias B
    (the priors are B^-1 of the camera positions' measurements) and 15 ground
    control points (point priors at their true positions) fixing the frame."""
    scene = syn.aerial_scene(seed=seed, nx=8, ny=8, n_points=3000, offset=(0.0, 0.0, 0.0),
                             gps_sigma=(0.2, 0.2, 0.4))
    w, t, s = np.array([0.01, -0.02, 0.015]), np.array([3.0, -2.0, 1.5]), 1.02
    R = syn.rotation_matrix(w)
    scene.extras["gps"] = ((scene.extras["gps"] - t) / s) @ R  # B^-1(p) = R^T (p - t) / s
    rng = np.random.default_rng(seed + 1)
    idx = rng.choice(len(scene.points), 15, replace=False)
    priors = (idx, scene.extras["true_points"][idx], np.full((15, 3), 0.05))
    return scene, (w, t, s), priors


def test_oracle_recovers_a_gps_bias():
    scene, (w, t, s), priors = biased_aerial()
    sol = oracle.solve(scene, loss=("HuberLoss", 2.0), irls="none", max_iterations=60, gps=True,
                       constant_cameras=True, bias=(np.zeros(3), np.zeros(3), 1.0, range(7)),
                       point_priors=priors)
    b = sol["bias"]
    assert np.abs(b[:3] - w).max() < 2e-3
    assert np.abs(b[3:6] - t).max() < 0.3
    assert abs(b[6] - s) < 2e-3
