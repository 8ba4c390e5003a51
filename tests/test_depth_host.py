"""Depth priors on observations (host side, no GPU).

RelativeDepthError (opensfm/src/lib/bundle/error/relative_depth_error.h):
the observed point in the camera frame -- the rig instance pose, then the
rig camera pose when it is used (WorldToCameraCoordinatesRig) -- gives a
depth, its z or, when radial, its distance to the camera, and the residual
(depth - value) / std.  The reference has no test of this term, so the
oracle's residual is checked against a numpy restatement and its Jacobian
against FP64 central differences; the adder's argument checks and the run's
refusal of a non-finite depth (bundle_adjuster.cc:582-586) follow.
"""
import numpy as np
import pytest

from opensfm_gb300 import pybundle, pygeometry
from opensfm_gb300 import synthetic as syn
from oracle import oracle


def _depth_np(inst, rig, X, value, std, radial):
    p = syn.world_to_camera(np.asarray(inst)[None], np.asarray(X)[None])[0]
    if rig is not None:
        p = syn.world_to_camera(np.asarray(rig)[None], p[None])[0]
    d = np.linalg.norm(p) if radial else p[2]
    return (d - value) / std


CASES = [(radial, rig) for radial in (True, False) for rig in (False, True)]


@pytest.mark.parametrize("radial,use_rig", CASES)
def test_depth_residual_matches_numpy_and_central_differences(radial, use_rig):
    rng = np.random.default_rng(3 + 2 * radial + use_rig)
    inst = np.concatenate([rng.normal(0, 0.4, 3), rng.normal(0, 2.0, 3)])
    rig = np.concatenate([rng.normal(0, 0.2, 3), rng.normal(0, 0.3, 3)]) if use_rig else None
    X = rng.normal(0, 3.0, 3) + np.array([0, 0, 8.0])
    value, std = 7.5, 0.25
    r, ji, jr, jp = oracle.depth_residual(inst, X, value, std, radial, rig)
    assert r == pytest.approx(_depth_np(inst, rig, X, value, std, radial), rel=1e-13, abs=1e-13)
    h = 1e-6

    def fd(vec, k, fn):
        a, b = vec.copy(), vec.copy()
        a[k] += h
        b[k] -= h
        return (fn(a) - fn(b)) / (2 * h)

    for k in range(6):
        assert ji[k] == pytest.approx(fd(inst, k, lambda v: _depth_np(v, rig, X, value, std, radial)), abs=2e-7)
        if use_rig:
            assert jr[k] == pytest.approx(fd(rig, k, lambda v: _depth_np(inst, v, X, value, std, radial)), abs=2e-7)
        else:
            assert jr[k] == 0.0
    for k in range(3):
        assert jp[k] == pytest.approx(fd(X, k, lambda v: _depth_np(inst, rig, v, value, std, radial)), abs=2e-7)


def test_oracle_solve_with_depth_priors_fixes_the_scale():
    # Without GPS the ring has a seven-dimensional gauge, scale included;
    # depth priors at the true depths pin the scale: the solved camera
    # distances then match the true ones.
    scene = syn.ring_scene(n_points=400, seed=9)
    depth = syn.depth_priors(scene, fraction=0.5, std=0.01, noise=0.0, seed=1)
    sol = oracle.solve(scene, loss=("HuberLoss", 1.0), irls="none", max_iterations=60, gps=False, depth=depth)
    c_true = scene.extras["true_poses"][:, 3:]
    c = sol["instances"][:, 3:]
    d_true = np.linalg.norm(c_true[0] - c_true[10])
    d_got = np.linalg.norm(c[0] - c[10])
    assert abs(d_got - d_true) / d_true < 5e-3
    assert sol["final_cost"] < sol["initial_cost"]


def _toy():
    ba = pybundle.BundleAdjuster()
    cam = pygeometry.Camera.create_perspective(1.0, 0.0, 0.0)
    ba.add_camera("cam1", cam, cam, True)
    ba.add_rig_camera("rig", pygeometry.Pose(), pygeometry.Pose(), True)
    ba.add_rig_instance("1", pygeometry.Pose(), {"s1": "cam1"}, {"s1": "rig"}, False)
    ba.add_point("p", np.array([0.0, 0.0, 5.0]), False)
    return ba


def test_depth_prior_argument_checks():
    ba = _toy()
    ba.add_point_projection_observation("s1", "p", np.zeros(2), 1.0, False,
                                        depth_prior=pybundle.Depth(5.0, True, 0.1))
    with pytest.raises(IndexError):
        ba.set_depth_priors([1], [5.0], [0.1])       # no second observation
    for sd in (0.0, -1.0, float("nan")):
        with pytest.raises(RuntimeError, match="std deviation must be positive"):
            ba.set_depth_priors([0], [5.0], [sd])


@pytest.mark.parametrize("bad", [float("nan"), float("inf"), 1e300])
def test_non_finite_depth_fails_at_run(bad):
    # AddRelativeDepthError throws "<shot> has non-finite depth prior" when
    # Run adds the block (bundle_adjuster.cc:582-586); 1e300 overflows the
    # float map::Depth holds.  The check runs before any device work.
    ba = _toy()
    ba.add_point_projection_observation("s1", "p", np.zeros(2), 1.0, False,
                                        depth_prior=pybundle.Depth(bad, False, 0.1))
    with pytest.raises(RuntimeError, match="s1 has non-finite depth prior"):
        ba.run()
