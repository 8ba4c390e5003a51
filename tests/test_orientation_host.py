"""Absolute orientation constraints on the host (no GPU): the library's
residuals and Jacobians (UpVectorError, PanAngleError, TiltAngleError,
RollAngleError of bundle/error/absolute_motion_errors.h:10-126, composed
through ShotRotationFunctor, position_functors.h:40-63) against the
oracle's independent restatement (rotation matrices instead of
quaternions) and central differences, and the closed forms of
opensfm/geometry.py:26-53 (pan/tilt/roll of a rotation)."""
import numpy as np
import pytest

from oracle import oracle
from opensfm_gb300 import pybundle


def _rot(a):
    a = np.asarray(a, np.float64)
    t = np.linalg.norm(a)
    if t < 1e-300:
        return np.eye(3)
    k = a / t
    K = np.array([[0, -k[2], k[1]], [k[2], 0, -k[0]], [-k[1], k[0], 0]])
    return np.eye(3) + np.sin(t) * K + (1 - np.cos(t)) * K @ K


def _cases():
    rng = np.random.default_rng(11)
    out = []
    for i in range(40):
        ri = rng.normal(size=3) * rng.choice([1e-9, 0.3, 1.5, 2.9])
        rc = None if i % 3 == 0 else rng.normal(size=3) * rng.choice([0.0, 0.2, 1.0])
        out.append((ri, rc))
    return out


KINDS = [("up_vector", [0.1, -0.9, 0.3], 0.05), ("pan", 0.7, 0.1), ("tilt", -0.4, 0.2), ("roll", 0.15, 0.3)]


@pytest.mark.parametrize("kind,target,std", KINDS)
def test_matches_oracle_and_finite_differences(kind, target, std):
    for ri, rc in _cases():
        r, J = pybundle.orientation_residual(kind, target, std, ri, rc)
        ro, Jo = oracle.orientation_residual(kind, target, std, ri, rc)
        np.testing.assert_allclose(r, ro, rtol=1e-9, atol=1e-9)
        np.testing.assert_allclose(J, Jo, rtol=1e-7, atol=1e-7)
        # central differences of the library's residuals, away from a
        # vertical optical axis where the angles are not differentiable
        z = (_rot(ri) @ _rot(np.zeros(3) if rc is None else rc))[:, 2]
        if kind != "up_vector" and np.linalg.norm(z[:2]) < 1e-3:
            continue
        x0 = np.concatenate([ri, np.zeros(3) if rc is None else rc])
        h = 1e-6
        for k in range(6 if rc is not None else 3):
            xp, xm = x0.copy(), x0.copy()
            xp[k] += h
            xm[k] -= h
            rp, _ = pybundle.orientation_residual(kind, target, std, xp[:3], xp[3:] if rc is not None else None)
            rm, _ = pybundle.orientation_residual(kind, target, std, xm[:3], xm[3:] if rc is not None else None)
            if np.abs(rp - rm).max() > 1.0:  # an angle wrapped across +-pi
                continue
            np.testing.assert_allclose((rp - rm) / (2 * h), J[:, k], rtol=1e-5, atol=1e-5 / std)


def test_angles_of_a_known_rotation():
    # cam-to-world rotation R: pan = atan2(R ez [0], R ez [1]),
    # tilt = atan2(-(R ez)[2], |(R ez)[:2]|), roll = asin of the x axis
    # out of the horizontal plane (geometry.py:36-53)
    rng = np.random.default_rng(3)
    for _ in range(20):
        a = rng.normal(size=3)
        R = _rot(a)
        z, x = R[:, 2], R[:, 0]
        pan = np.arctan2(z[0], z[1])
        tilt = np.arctan2(-z[2], np.linalg.norm(z[:2]))
        h = np.cross(z, [0, 0, 1])
        h /= np.linalg.norm(h)
        roll = np.arcsin(np.dot(z, np.cross(x, h)))
        for kind, want in (("pan", pan), ("tilt", tilt), ("roll", roll)):
            r, _ = pybundle.orientation_residual(kind, want, 1.0, a)
            assert abs(r[0]) < 1e-12, (kind, r)
        # the up vector that R takes to +z is the third row of R
        r, _ = pybundle.orientation_residual("up_vector", R[2] * 3.0, 0.5, a)
        np.testing.assert_allclose(r, 0, atol=1e-12)


def test_rig_camera_composition():
    # the shot rotation is R(instance) R(rig camera)
    rng = np.random.default_rng(5)
    for _ in range(10):
        ri, rc = rng.normal(size=3), rng.normal(size=3)
        R = _rot(ri) @ _rot(rc)
        z = R[:, 2]
        r, _ = pybundle.orientation_residual("pan", np.arctan2(z[0], z[1]), 1.0, ri, rc)
        assert abs(r[0]) < 1e-12


def test_degenerate_and_invalid():
    # pan is zero when the optical axis is vertical
    r, J = pybundle.orientation_residual("pan", 0.3, 1.0, np.zeros(3))
    assert r[0] == 0.0 and np.all(J == 0.0)
    with pytest.raises(pybundle._lib.GbbaError):
        pybundle.orientation_residual("pan", 0.3, 0.0, np.zeros(3))
    with pytest.raises(pybundle._lib.GbbaError):
        pybundle.orientation_residual("up_vector", [0, 0, 0], 1.0, np.zeros(3))
