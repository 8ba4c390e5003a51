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


# ---- constraints between shots (relative_motion_errors.h:66-126,
# motion_prior_errors.h:12-74)

def _relative_cases(n_shots, seed):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(30):
        poses = np.concatenate([rng.normal(size=(n_shots, 3)) * 0.8, rng.normal(size=(n_shots, 3)) * 3], axis=1)
        rig = None
        if i % 2:
            rig = np.concatenate([rng.normal(size=(n_shots, 3)) * 0.3, rng.normal(size=(n_shots, 3))], axis=1)
        out.append((poses, rig))
    return out


REL = [
    ("relative_rotation", 2, lambda rng: np.concatenate([rng.normal(size=3) * 0.5,
                                                         (np.eye(3) + 0.1 * rng.normal(size=(3, 3))).ravel()])),
    ("common_position", 2, lambda rng: np.array([0.5, 0.2])),
    ("linear_motion", 3, lambda rng: np.array([0.4, 0.3, 0.05])),
    ("gauge_scale", 2, lambda rng: np.array([2.5])),
]


@pytest.mark.parametrize("kind,n_shots,make_params", REL)
def test_relative_matches_oracle_and_finite_differences(kind, n_shots, make_params):
    rng = np.random.default_rng(7)
    for poses, rig in _relative_cases(n_shots, 3):
        prm = make_params(rng)
        r, J = pybundle.relative_residual(kind, poses, prm, rig)
        ro, Jo = oracle.relative_residual(kind, poses, prm, rig)
        np.testing.assert_allclose(r, ro, rtol=1e-9, atol=1e-9)
        np.testing.assert_allclose(J, Jo, rtol=1e-7, atol=1e-7)
        # central differences of the library's residuals over every slot
        x0 = np.concatenate([poses, np.zeros_like(poses) if rig is None else rig], axis=1)  # [n][12]
        h = 1e-6
        for k in range(n_shots):
            for a in range(12 if rig is not None else 6):
                xp, xm = x0.copy(), x0.copy()
                xp[k, a] += h
                xm[k, a] -= h
                rp, _ = pybundle.relative_residual(kind, xp[:, :6], prm, xp[:, 6:] if rig is not None else None)
                rm, _ = pybundle.relative_residual(kind, xm[:, :6], prm, xm[:, 6:] if rig is not None else None)
                np.testing.assert_allclose((rp - rm) / (2 * h), J[:, 12 * k + a], rtol=1e-5, atol=2e-5)


def test_relative_known_values():
    # relative rotation: zero when R_ij R_i^T R_j = I, i.e. R_ij is the
    # inverse of R_i^T R_j; common position: zero within the margin; linear
    # motion:
    # zero for shot 1 on the segment at fraction alpha with the rotation
    # interpolated
    rng = np.random.default_rng(9)
    ri, rj = rng.normal(size=3) * 0.4, rng.normal(size=3) * 0.4
    M = _rot(ri).T @ _rot(rj)
    th = np.arccos(np.clip((np.trace(M) - 1) / 2, -1, 1))
    rij = th / (2 * np.sin(th)) * np.array([M[2, 1] - M[1, 2], M[0, 2] - M[2, 0], M[1, 0] - M[0, 1]])
    poses = np.array([np.r_[ri, 0, 0, 0], np.r_[rj, 1, 2, 3]])
    r, _ = pybundle.relative_residual("relative_rotation", poses, np.r_[-rij, np.eye(3).ravel()])
    np.testing.assert_allclose(r, 0, atol=1e-12)
    poses = np.array([np.r_[0, 0, 0, 1.0, 2.0, 3.0], np.r_[0, 0, 0, 1.3, 1.8, 4.0]])
    r, _ = pybundle.relative_residual("common_position", poses, [0.5, 0.25])
    np.testing.assert_allclose(r, [0, 0, -4.0], atol=1e-12)
    p0, p2 = np.array([0.0, 0, 0]), np.array([4.0, 2, -2])
    poses = np.array([np.r_[0, 0, 0, p0], np.r_[0, 0, 0.25 * 0.8, 0.25 * p2], np.r_[0, 0, 0.8, p2]])
    r, _ = pybundle.relative_residual("linear_motion", poses, [0.25, 1.0, 1.0])
    np.testing.assert_allclose(r, 0, atol=1e-12)


def _bell(size, r, mu_x, mu_y):
    # the cost surface of test_bundle.py:675-693: 1 - a normalised Gaussian
    x, y = np.meshgrid(np.linspace(-r, r, size), np.linspace(r, -r, size))
    z = np.exp(-((x - mu_x) ** 2 / (2 * (r / 2) ** 2) + (y - mu_y) ** 2 / (2 * (r / 2) ** 2)))
    return 1 - z / z.max()


def test_heatmap_matches_oracle_and_finite_differences():
    size, rad = 41, 10.0
    res = 2 * rad / (size - 1)
    grid = _bell(size, rad, 1.0, -1.0)
    rng = np.random.default_rng(2)
    for i in range(40):
        pose = np.r_[rng.normal(size=3) * 0.5, rng.uniform(-13, 13, 2), rng.normal()]
        rig = None if i % 2 else np.r_[rng.normal(size=3) * 0.3, rng.normal(size=3)]
        xo, yo, std = rng.normal(size=2).tolist() + [0.7]
        r, J = pybundle.heatmap_residual(grid, size, res, xo, yo, std, pose, rig)
        ro, Jo = oracle.heatmap_residual(grid, size, res, xo, yo, std, pose, rig)
        assert abs(r - ro) < 1e-12
        np.testing.assert_allclose(J, Jo, atol=1e-10)
        h = 1e-6
        x0 = np.r_[pose, np.zeros(6) if rig is None else rig]
        for k in range(12 if rig is not None else 6):
            xp, xm = x0.copy(), x0.copy()
            xp[k] += h
            xm[k] -= h
            rp, _ = pybundle.heatmap_residual(grid, size, res, xo, yo, std, xp[:6], xp[6:] if rig is not None else None)
            rm, _ = pybundle.heatmap_residual(grid, size, res, xo, yo, std, xm[:6], xm[6:] if rig is not None else None)
            if abs(rp - rm) > 0:  # the spline is C1: central differences agree except across clamped borders
                assert abs((rp - rm) / (2 * h) - J[k]) < 1e-4, (k, (rp - rm) / (2 * h), J[k])


def test_heatmap_interpolates_grid_nodes():
    # at a node the spline returns the node's value
    grid = np.arange(35, dtype=np.float64).reshape(5, 7) ** 1.5
    res = 0.5
    for i in range(1, 4):
        for j in range(1, 6):
            # row = height / 2 - y / res, col = width / 2 + x / res
            x = (j - 3.5) * res
            y = (2.5 - i) * res
            r, _ = pybundle.heatmap_residual(grid, 7, res, 0.0, 0.0, 1.0, np.r_[0, 0, 0, x, y, 0])
            assert abs(r - grid[i, j]) < 1e-12


def test_relative_motion_matches_oracle_and_finite_differences():
    # RelativeMotionError (relative_motion_errors.h:13-64): instance poses
    # only (rig cameras unused), the two scales in columns 24 and 25
    rng = np.random.default_rng(12)
    for i in range(30):
        poses = np.concatenate([rng.normal(size=(2, 3)) * 0.7, rng.normal(size=(2, 3)) * 3], axis=1)
        motion = np.r_[rng.normal(size=3) * 0.4, rng.normal(size=3), rng.uniform(0.5, 2)]
        observed = float(i % 2)
        M = np.eye(7) + 0.1 * rng.normal(size=(7, 7))
        sc = rng.uniform(0.3, 3.0, 2)
        prm = np.r_[motion, observed, M.ravel(), sc]
        r, J = pybundle.relative_residual("relative_motion", poses, prm)
        ro, Jo = oracle.relative_residual("relative_motion", poses, np.r_[motion, observed, M.ravel()], scales=sc)
        np.testing.assert_allclose(r, ro, rtol=1e-9, atol=1e-9)
        np.testing.assert_allclose(J, Jo, rtol=1e-7, atol=1e-7)
        assert np.all(J[:, 6:12] == 0) and np.all(J[:, 18:24] == 0) and np.all(J[:, 26:] == 0)
        h = 1e-6
        for col in list(range(6)) + list(range(12, 18)) + [24, 25]:
            dp, ds = poses.copy(), sc.copy()
            if col < 24:
                dp[col // 12, col % 12] += h
            else:
                ds[col - 24] += h
            rp, _ = pybundle.relative_residual("relative_motion", dp, np.r_[motion, observed, M.ravel(), ds])
            dp, ds = poses.copy(), sc.copy()
            if col < 24:
                dp[col // 12, col % 12] -= h
            else:
                ds[col - 24] -= h
            rm, _ = pybundle.relative_residual("relative_motion", dp, np.r_[motion, observed, M.ravel(), ds])
            np.testing.assert_allclose((rp - rm) / (2 * h), J[:, col], rtol=1e-5, atol=2e-5)
    # a zero scale leaves the residual undefined, as the functor fails
    r, _ = pybundle.relative_residual("relative_motion", np.zeros((2, 6)), np.r_[np.zeros(7), 0, np.eye(7).ravel(),
                                                                                 0.0, 1.0])
    assert np.all(np.isnan(r))


def test_relative_motion_known_value():
    # test_bundle.py:167-194: instances at (0,0,0) and (2,0,0), identity
    # rotations, t_ij = (-1, 0, 0): zero residual at s_j = 0.5
    poses = np.array([[0, 0, 0, 0, 0, 0], [0, 0, 0, 2, 0, 0]], np.float64)
    prm = np.r_[0, 0, 0, -1, 0, 0, 1, 0, np.eye(7).ravel(), 4.0, 0.5]
    r, _ = pybundle.relative_residual("relative_motion", poses, prm)
    np.testing.assert_allclose(r, 0, atol=1e-15)


def test_host_losses_match_the_oracle():
    # the losses of the relative rotations and motions (host FP64) against
    # the oracle's projection losses (Ceres' documented forms), and Tukey's
    # closed form (the common-position loss)
    import ctypes as C
    from opensfm_gb300 import _lib
    L = _lib.lib()
    f = L.gbba_host_loss
    f.argtypes = [C.c_int, C.c_double, C.c_double, C.POINTER(C.c_double)]
    f.restype = C.c_int

    def host(kind, a, s):
        rho = (C.c_double * 3)()
        assert f(kind, a, s, rho) == 0
        return np.array(rho[:])

    for kind in range(5):
        for a in (0.5, 1.0, 2.0):
            for s in (0.0, 0.1, 0.9, 1.0, 3.0, 40.0):
                np.testing.assert_allclose(host(kind, a, s), oracle.loss(kind, a, s), rtol=1e-12, atol=1e-300)
    for a in (0.5, 1.0, 2.0):
        for s in (0.0, 0.1, 0.9, 3.0, 40.0):
            b = a * a
            v = 1 - s / b
            want = [b / 3 * (1 - v ** 3), v * v, -2 * v / b] if s <= b else [b / 3, 0.0, 0.0]
            np.testing.assert_allclose(host(5, a, s), want, rtol=1e-12, atol=1e-300)
