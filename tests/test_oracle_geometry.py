"""The FP64 oracle against the reference's own known answers.

Golden pixels: opensfm/src/lib/geometry/test/camera_test.cc:119-172.
Analytic vs autodiff camera Jacobians (tolerance 1e-12):
  geometry/test/camera_functions_test.cc:232-431 (fixture :236-249).
PoseFunctor vs autodiff (tolerance 1e-15): camera_functions_test.cc:142-229.
Reprojection residual Jacobians vs autodiff (tolerance 1e-14):
  bundle/test/reprojection_errors_test.cc:23-280.
The reference's Eigen AutoDiffScalar is replaced by the oracle's own dual
numbers; FP64 central differences are an extra, independent check.
"""
import numpy as np
import pytest

from oracle import oracle
from opensfm_gb300.scene import (BROWN, DUAL, FISHEYE, FISHEYE62, FISHEYE624, FISHEYE_OPENCV,
                                 PERSPECTIVE, RADIAL, SIMPLE_RADIAL, SPHERICAL)

FOCAL = 0.4
PP = (0.1, -0.05)
DIST = (-0.1, 0.03)
DIST_BROWN = (-0.1, 0.03, 0.001, 0.001, 0.002)
DIST_FISHEYE = (-0.1, 0.03, 0.001, 0.005)
DIST_F62 = (-0.1, 0.03, 0.001, 0.005, 0.02, 0.001, 0.0007, -0.01)
DIST_F624 = DIST_F62 + (0.01, -0.007, -0.03, 0.0053)
DIST_RADIAL = (0.1, 0.03)

# geometry::Camera parameter vectors (camera.cc:11-172) of the derivative fixture.
FIXTURE_CAMERAS = {
    PERSPECTIVE: (-0.1, 0.01, FOCAL),
    FISHEYE: (-0.1, 0.01, FOCAL),
    FISHEYE_OPENCV: DIST_FISHEYE + (FOCAL, 0.9) + PP,
    FISHEYE62: DIST_F62 + (FOCAL, 1.0) + PP,
    FISHEYE624: DIST_F624 + (FOCAL, 1.0) + PP,
    RADIAL: DIST_RADIAL + (FOCAL, 1.0) + PP,
    SIMPLE_RADIAL: (DIST_RADIAL[0], FOCAL, 1.0) + PP,
    BROWN: DIST_BROWN + (FOCAL, 0.9) + PP,
    DUAL: (0.5, -0.1, 0.01, FOCAL),
}
POINT = np.array([0.1, 0.2, 0.3])


@pytest.mark.parametrize("with_tangential", [False, True])
def test_fisheye624_golden_pixels(with_tangential):
    # camera_test.cc:119-172 (pixel-unit focal and principal point)
    width, height = 200, 100
    f = width / (2 * np.pi)
    pts = np.array([[10.0, 0.0, 0.0], [0.0, 10.0, 0.0], [1e-6, 1e-6, 10.0]])
    if with_tangential:
        dist = (0, 0, 0, 0, 0, 0, 0.03, 0.01, 0.01, -0.007, -0.03, 0.0053)
        golden = np.array([[151.7850648, 51.02708265], [100.2142719, 105.7394678], [100.0, 50.0]])
    else:
        dist = (0, 0, 0, 0, 0, 0, 0, 0, 0.01, -0.007, -0.03, 0.0053)
        golden = np.array([[149.42887062, 48.67088846], [99.4288738, 98.67088528], [100.0, 50.0]])
    params = np.array(dist + (f, 1.0, width / 2, height / 2))
    got = np.array([oracle.project(FISHEYE624, p, params)[0] for p in pts])
    # Eigen isApprox(.., 1e-5): relative Frobenius-norm closeness
    assert np.linalg.norm(got - golden) <= 1e-5 * min(np.linalg.norm(got), np.linalg.norm(golden))


@pytest.mark.parametrize("model", sorted(FIXTURE_CAMERAS))
def test_camera_jacobian_matches_autodiff(model):
    params = np.array(FIXTURE_CAMERAS[model])
    uv, jp, jc = oracle.project(model, POINT, params)
    uv_ad, jp_ad, jc_ad = oracle.project(model, POINT, params, ad=True)
    np.testing.assert_allclose(uv, uv_ad, atol=1e-12, rtol=0)
    np.testing.assert_allclose(jp, jp_ad, atol=1e-12, rtol=0)
    np.testing.assert_allclose(jc, jc_ad, atol=1e-12, rtol=0)


@pytest.mark.parametrize("model", sorted(FIXTURE_CAMERAS))
def test_camera_jacobian_matches_central_differences(model):
    params = np.array(FIXTURE_CAMERAS[model], np.float64)
    _, jp, jc = oracle.project(model, POINT, params)
    h = 1e-6
    for j in range(3):
        d = np.zeros(3)
        d[j] = h
        fd = (oracle.project(model, POINT + d, params)[0] - oracle.project(model, POINT - d, params)[0]) / (2 * h)
        np.testing.assert_allclose(jp[:, j], fd, atol=1e-7, rtol=1e-6)
    for j in range(len(params)):
        d = np.zeros(len(params))
        d[j] = h
        fd = (oracle.project(model, POINT, params + d)[0] - oracle.project(model, POINT, params - d)[0]) / (2 * h)
        np.testing.assert_allclose(jc[:, j], fd, atol=1e-7, rtol=1e-6)


def _rodrigues(aa):
    th = np.linalg.norm(aa)
    k = aa / th
    K = np.array([[0, -k[2], k[1]], [k[2], 0, -k[0]], [-k[1], k[0], 0]])
    return np.eye(3) + np.sin(th) * K + (1 - np.cos(th)) * K @ K


def test_pose_functor_forward_and_jacobian():
    # camera_functions_test.cc:142-229: point (1,2,3), rt (0.1..0.6)
    X = np.array([1.0, 2.0, 3.0])
    rt = np.array([0.1, 0.2, 0.3, 0.4, 0.5, 0.6])
    out, J = oracle.pose_jacobian(X, rt)
    expected = _rodrigues(-rt[:3]) @ (X - rt[3:])
    np.testing.assert_allclose(out, expected, atol=1e-15, rtol=0)
    _, J_ad = oracle.pose_jacobian(X, rt, ad=True)
    np.testing.assert_allclose(J, J_ad, atol=1e-15, rtol=0)


def test_pose_functor_small_angle_branch():
    # theta^2 below machine epsilon takes the first-order branch
    X = np.array([1.0, -2.0, 0.5])
    rt = np.array([1e-9, -2e-9, 3e-9, 0.1, 0.2, 0.3])
    out, J = oracle.pose_jacobian(X, rt)
    _, J_ad = oracle.pose_jacobian(X, rt, ad=True)
    np.testing.assert_allclose(out, (X - rt[3:]) + np.cross(-rt[:3], X - rt[3:]), atol=1e-15)
    np.testing.assert_allclose(J, J_ad, atol=1e-12)


# reprojection_errors_test.cc:130-190 camera vectors
RESIDUAL_CAMERAS = {
    BROWN: (0.3, 1.0, 0.001, -0.02, 0.1, -0.03, 0.001, -0.005, 0.001),
    PERSPECTIVE: (0.3, 0.1, -0.03),
    FISHEYE: (0.3, 0.1, -0.03),
    FISHEYE_OPENCV: (0.3, 1.0, 0.001, -0.02, 0.1, -0.03, 0.001, -0.005),
    FISHEYE62: (0.3, 1.0, 0.001, -0.02, 0.1, -0.03, 0.001, -0.005, 0.01, 0.006, 0.02, 0.003),
    FISHEYE624: (0.3, 1.0, 0.001, -0.02, 0.1, -0.03, 0.001, -0.005, 0.01, 0.006, 0.02, 0.003, 0.001,
                 -0.009, -0.01, 0.03),
    DUAL: (0.5, 0.3, 0.1, -0.03),
}
RT = np.array([0.1, 0.2, 0.3, 0.4, 0.5, 0.6])
XPT = np.array([1.0, 2.0, 3.0])
OBS = np.array([0.5, 0.5])
STD = 0.1


@pytest.mark.parametrize("model", sorted(RESIDUAL_CAMERAS))
@pytest.mark.parametrize("rig", [True, False])
def test_reprojection_jacobian_matches_autodiff(model, rig):
    cam = np.array(RESIDUAL_CAMERAS[model])
    rig_pose = RT if rig else None
    a = oracle.residual_jacobian(model, cam, RT, rig_pose, XPT, OBS, STD)
    b = oracle.residual_jacobian(model, cam, RT, rig_pose, XPT, OBS, STD, ad=True)
    for x, y in zip(a, b):
        np.testing.assert_allclose(x, y, atol=1e-14 * max(1.0, np.abs(y).max()), rtol=0)


@pytest.mark.parametrize("rig", [True, False])
def test_spherical_residual_matches_autodiff(rig):
    # reprojection_errors_test.cc:192-280
    a = oracle.residual_jacobian(SPHERICAL, [0.0], RT, RT if rig else None, XPT, OBS, STD)
    b = oracle.residual_jacobian(SPHERICAL, [0.0], RT, RT if rig else None, XPT, OBS, STD, ad=True)
    assert a[0].shape == (3,)
    for x, y in zip(a, b):
        np.testing.assert_allclose(x, y, atol=1e-14 * max(1.0, np.abs(y).max()), rtol=0)
    # the camera block of a spherical residual is zero
    assert np.all(a[1] == 0.0)


@pytest.mark.parametrize("kind", [1, 2, 3, 4])
@pytest.mark.parametrize("s", [0.01, 0.7, 3.0, 40.0])
def test_loss_derivatives(kind, s):
    a = 1.3
    rho = oracle.loss(kind, a, s)
    h = 1e-6 * max(1.0, s)
    rp = oracle.loss(kind, a, s + h)
    rm = oracle.loss(kind, a, s - h)
    np.testing.assert_allclose(rho[1], (rp[0] - rm[0]) / (2 * h), rtol=1e-6, atol=1e-9)
    np.testing.assert_allclose(rho[2], (rp[1] - rm[1]) / (2 * h), rtol=1e-5, atol=1e-9)


def test_trivial_and_small_huber_are_identity():
    assert np.allclose(oracle.loss(0, 1.0, 2.5), [2.5, 1.0, 0.0])
    assert np.allclose(oracle.loss(1, 2.0, 1.0), [1.0, 1.0, 0.0])


def test_mixture_reweighting_separates_mixture():
    # bundle/test/reweighting_test.cc:131-160 (MixtureReweighting_SeparatesMixture):
    # 200 inliers at (0.1, 0.1), 20 outliers at (10, 10) starting at weight
    # 0.01, outlier density 0.1 -> inliers above 0.8, outliers below 0.1.
    res = np.array([[0.1, 0.1]] * 200 + [[10.0, 10.0]] * 20)
    w0 = np.array([1.0] * 200 + [0.01] * 20)
    ll, w = oracle.mixture_group(res, w0, 0.1)
    assert ll != 0.0
    assert w[0] > 0.8
    assert w[200] < 0.1


def test_mixture_reweighting_small_group_untouched():
    # groups below the minimum sample size (10) keep their weights
    # (mixture_reweighting.cc:22-24)
    res = np.full((9, 2), 5.0)
    ll, w = oracle.mixture_group(res, np.ones(9), 0.1)
    assert ll == 0.0 and np.all(w == 1.0)
