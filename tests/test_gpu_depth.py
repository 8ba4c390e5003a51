"""Depth priors on observations: GPU solves against the FP64 CPU oracle.

Every depth prior (RelativeDepthError, bundle/error/relative_depth_error.h,
added by AddRelativeDepthError at bundle_adjuster.cc:572-604) rides on a
slot of its own beside the observation's projection, so the record passes,
the Schur elimination of its point and the dense reduced system take it as
they take a projection.  Bar: final cost within 1e-6 of the oracle's (the
solver tests' bar), RMS reprojection within 1e-3 px, in FP64 and mixed
precision, on the PCG and the exact (dense) path, with radial and z depths,
under a composed rig camera and with IRLS mixture reweighting (group DEPTH).
"""
import numpy as np
import pytest

from oracle import oracle
from opensfm_gb300 import synthetic as syn
from opensfm_gb300.pybundle import adjuster_from_scene

pytestmark = pytest.mark.gpu


def _rms_px(errors, width=1000):
    e = errors[:, :2] * width
    return float(np.sqrt((e ** 2).sum(1).mean()))


def _case(radial=True, seed=9):
    scene = syn.ring_scene(n_points=1500, seed=seed)
    depth = syn.depth_priors(scene, fraction=0.3, std=0.05, radial=radial, noise=0.02, seed=seed + 1)
    return scene, depth


def _solve(scene, depth, precision, solver, **kw):
    pcg = 1e-10 if precision == "fp64" else 1e-4
    ba = adjuster_from_scene(scene, precision=precision, pcg_tolerance=pcg, linear_solver=solver, gps=False,
                             depth=depth, **kw)
    ba.run()
    errs, w, _ = ba.projection_results()
    return ba, errs, w


@pytest.mark.parametrize("radial", [True, False])
@pytest.mark.parametrize("solver", ["ITERATIVE_SCHUR", "SPARSE_SCHUR"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_depth_priors_match_oracle(precision, solver, radial):
    scene, depth = _case(radial)
    ref = oracle.solve(scene, loss=("HuberLoss", 1.0), irls="none", max_iterations=50, gps=False, depth=depth)
    ba, errs, _ = _solve(scene, depth, precision, solver, loss=("HuberLoss", 1.0), irls="none", max_iterations=50)
    s = ba.summary()
    assert s["usable"]
    rel = abs(s["final_cost"] - ref["final_cost"]) / ref["final_cost"]
    assert rel < 1e-6, (s["final_cost"], ref["final_cost"])
    # projection results stay one row per observation (depth slots are not
    # reprojection errors)
    assert errs.shape == (scene.n_observations, 3)
    assert abs(_rms_px(errs) - _rms_px(ref["errors"])) < 1e-3
    # the depth priors fix the scale but not the rotation and translation of
    # the gauge: FP64 takes the oracle's steps and ends at the same point of
    # it; mixed-precision PCG ends elsewhere on it, so its points are compared
    # by their distances to the first point (invariant under rigid motion)
    pts, ref_pts = ba.get_points(), ref["points"]
    if precision == "fp64" or solver == "SPARSE_SCHUR":
        np.testing.assert_allclose(pts, ref_pts, atol=1e-4)
    np.testing.assert_allclose(np.linalg.norm(pts - pts[0], axis=1), np.linalg.norm(ref_pts - ref_pts[0], axis=1),
                               atol=1e-3)


def test_depth_priors_with_a_composed_rig_camera():
    # a fixed rig camera that is not the identity is composed with every
    # shot (IsRigCameraUseful): the depth is taken in the rig camera's frame
    scene, depth = _case(radial=True, seed=13)
    rig = np.array([0.01, -0.02, 0.005, 0.05, 0.0, -0.03])
    ref = oracle.solve(scene, loss=("HuberLoss", 1.0), irls="none", max_iterations=50, gps=False, depth=depth,
                       rig_pose=rig)
    for precision, solver in (("fp64", "SPARSE_SCHUR"), ("mixed", "ITERATIVE_SCHUR")):
        ba, errs, _ = _solve(scene, depth, precision, solver, loss=("HuberLoss", 1.0), irls="none",
                             max_iterations=50, rig_pose=rig)
        rel = abs(ba.summary()["final_cost"] - ref["final_cost"]) / ref["final_cost"]
        assert rel < 1e-6, (precision, ba.summary()["final_cost"], ref["final_cost"])


def test_depth_priors_irls_mixture_matches_oracle():
    # the depth residuals form the IRLS group DEPTH (one-dimensional mixture)
    scene = syn.ring_scene(n_points=1500, outlier_ratio=0.02, seed=21)
    depth = syn.depth_priors(scene, fraction=0.4, std=0.05, noise=0.02, seed=22)
    # a few depth outliers for the DEPTH group to down-weight
    depth[1][::25] += 3.0
    ref = oracle.solve(scene, irls="mixture", max_iterations=100, gps=False, depth=depth)
    ba, errs, w = _solve(scene, depth, "fp64", "SPARSE_SCHUR", irls="mixture", max_iterations=100)
    rel = abs(ba.summary()["final_cost"] - ref["final_cost"]) / ref["final_cost"]
    assert rel < 1e-6, (ba.summary()["final_cost"], ref["final_cost"])
    assert np.abs(w - ref["weights"]).max() < 1e-3
    assert any(line.startswith("DEPTH") or "DEPTH" in line for line in ba.irls_report())


def test_depth_priors_matrix_free_follow_stored_records():
    scene, depth = _case(radial=False, seed=17)
    kw = dict(loss=("HuberLoss", 1.0), irls="none", max_iterations=20)
    stored, _, _ = _solve(scene, depth, "fp64", "ITERATIVE_SCHUR", matrix_free=-1, **kw)
    free, _, _ = _solve(scene, depth, "fp64", "ITERATIVE_SCHUR", matrix_free=1, **kw)
    t1, t2 = stored.trace(), free.trace()
    n = min(len(t1), len(t2))
    np.testing.assert_allclose(t2[:n, 1], t1[:n, 1], rtol=1e-9)
