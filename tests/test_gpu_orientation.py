"""Absolute orientation constraints (up vector, pan, tilt, roll) in the GPU
solve, against the FP64 CPU oracle and the reference's own singleton tests.

The constraints are host terms of the camera-side system (a few residuals
per shot under CauchyLoss(1), bundle_adjuster.cc:1011-1082); the GPU solve
adds their Gauss-Newton blocks to the implicit Schur product, the
block-Jacobi preconditioner and the dense reduced camera system.  Bars as
in test_gpu_solver.py: converged cost within 1e-6 relative of the oracle's.
"""
import numpy as np
import pytest

from oracle import oracle
from opensfm_gb300 import pybundle, pygeometry
from opensfm_gb300 import synthetic as syn
from opensfm_gb300.pybundle import adjuster_from_scene

pytestmark = pytest.mark.gpu


def _rot(a):
    a = np.asarray(a, np.float64)
    t = np.linalg.norm(a)
    if t < 1e-300:
        return np.eye(3)
    k = a / t
    K = np.array([[0, -k[2], k[1]], [k[2], 0, -k[0]], [-k[1], k[0], 0]])
    return np.eye(3) + np.sin(t) * K + (1 - np.cos(t)) * K @ K


def _ptr(R_wc):
    """Pan, tilt, roll of a world-to-camera rotation (opensfm/geometry.py:26-53)."""
    z = R_wc.T @ [0, 0, 1]
    x = R_wc.T @ [1, 0, 0]
    pan = np.arctan2(z[0], z[1])
    tilt = np.arctan2(-z[2], np.linalg.norm(z[:2]))
    a = np.cross(z, [0, 0, 1])
    a /= np.linalg.norm(a)
    roll = np.arcsin(np.dot(z, np.cross(x, a)))
    return pan, tilt, roll


def _singleton(precision):
    ba = pybundle.BundleAdjuster()
    ba.set_precision(precision)
    ba.set_skip_initial_reweighting(True)
    cam = pygeometry.Camera.create_perspective(1.0, 0.0, 0.0)
    ba.add_camera("cam1", cam, cam, True)
    ba.add_rig_camera("rig_cam1", pygeometry.Pose(), pygeometry.Pose(), True)
    ba.add_rig_instance("1", pygeometry.Pose(np.array([0.5, 0, 0]), np.array([0, 0, 0])), {"1": "cam1"},
                        {"1": "rig_cam1"}, False)
    ba.add_rig_instance_position_prior("1", np.array([1, 0, 0]), np.array([1, 1, 1]), "")
    return ba


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_singleton_up_vector_and_pan(precision):
    # test_bundle.py:47-65
    ba = _singleton(precision)
    ba.add_absolute_up_vector("1", np.array([0, -1, 0]), 1)
    ba.add_absolute_pan("1", np.radians(180), 1)
    ba.run()
    s1 = ba.get_rig_instance_pose("1")
    assert np.allclose(s1.translation, [1, 0, 0], atol=1e-6), s1.translation


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_singleton_pan_tilt_roll(precision):
    # test_bundle.py:68-92
    pan, tilt, roll = 1, 0.3, 0.2
    ba = _singleton(precision)
    ba.add_absolute_pan("1", pan, 1)
    ba.add_absolute_tilt("1", tilt, 1)
    ba.add_absolute_roll("1", roll, 1)
    ba.run()
    pose = ba.get_rig_instance_pose("1")
    assert np.allclose(pose.get_origin(), [1, 0, 0], atol=1e-6)
    assert np.allclose(_ptr(pose.get_rotation_matrix()), (pan, tilt, roll)), _ptr(pose.get_rotation_matrix())


def _constraints(scene, seed=0, outliers=0):
    """Constraints on every shot from its initial rotation, perturbed by
    0.02 rad (angles) / 0.02 (up vector); `outliers` shots get a pan 1 rad
    off."""
    rng = np.random.default_rng(seed)
    out = []
    for s in range(len(scene.shot_camera)):
        R = _rot(scene.rig_instance_poses[int(scene.shot_rig_instance[s])][:3])  # camera to world
        z, x = R[:, 2], R[:, 0]
        pan = np.arctan2(z[0], z[1])
        tilt = np.arctan2(-z[2], np.linalg.norm(z[:2]))
        h = np.cross(z, [0, 0, 1])
        h /= np.linalg.norm(h)
        roll = np.arcsin(np.dot(z, np.cross(x, h)))
        up = R[2] + rng.normal(0, 0.02, 3)
        out.append(("up_vector", s, up, 0.05))
        out.append(("pan", s, pan + rng.normal(0, 0.02) + (1.0 if s < outliers else 0.0), 0.05))
        out.append(("tilt", s, tilt + rng.normal(0, 0.02), 0.05))
        out.append(("roll", s, roll + rng.normal(0, 0.02), 0.05))
    return out


def _add(ba, constraints):
    for kind, s, v, std in constraints:
        if kind == "up_vector":
            ba.add_absolute_up_vector(str(s), np.asarray(v), std)
        else:
            getattr(ba, "add_absolute_" + kind)(str(s), float(v), std)


@pytest.mark.parametrize("solver", ["ITERATIVE_SCHUR", "SPARSE_SCHUR"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_ring_orientation_matches_oracle(precision, solver):
    scene = syn.ring_scene(n_points=1500, seed=9)
    cons = _constraints(scene, seed=1)
    ref = oracle.solve(scene, loss=("HuberLoss", 1.0), irls="none", max_iterations=60, gps=False, orientation=cons)
    free = oracle.solve(scene, loss=("HuberLoss", 1.0), irls="none", max_iterations=60, gps=False)
    assert ref["final_cost"] > free["final_cost"] * 1.0001  # the constraints pull against the images
    ba = adjuster_from_scene(scene, precision=precision, loss=("HuberLoss", 1.0), irls="none", max_iterations=60,
                             gps=False, linear_solver=solver, pcg_tolerance=1e-10 if precision == "fp64" else 1e-4)
    _add(ba, cons)
    ba.run()
    s = ba.summary()
    assert s["usable"]
    rel = abs(s["final_cost"] - ref["final_cost"]) / ref["final_cost"]
    assert rel < 1e-6, (s["final_cost"], ref["final_cost"])
    # the constraints fix the rotation gauge: same rotations as the oracle
    got = np.stack([ba.get_rig_instance_pose(str(i)).rotation for i in range(len(scene.shot_camera))])
    want = np.stack([pygeometry.Pose.from_ba_data(p).rotation for p in ref["instances"]])
    np.testing.assert_allclose(got, want, atol=1e-4)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_ring_orientation_irls_mixture_matches_oracle(precision):
    # 20 constraints of each kind: every group is reweighted; 3 pans are
    # gross outliers
    scene = syn.ring_scene(n_points=1500, outlier_ratio=0.03, seed=5)
    cons = _constraints(scene, seed=2, outliers=3)
    ref = oracle.solve(scene, irls="mixture", max_iterations=100, gps=False, orientation=cons)
    # exact (dense) steps: the reweighting states track the oracle's path
    ba = adjuster_from_scene(scene, precision=precision, irls="mixture", max_iterations=100, gps=False,
                             linear_solver="SPARSE_SCHUR")
    _add(ba, cons)
    ba.run()
    s = ba.summary()
    assert s["usable"]
    rel = abs(s["final_cost"] - ref["final_cost"]) / ref["final_cost"]
    assert rel < (1e-6 if precision == "fp64" else 1e-5), (s["final_cost"], ref["final_cost"])


def test_batch_rejects_orientation_constraints():
    scene = syn.ring_scene(n_points=300, seed=3)
    ba = adjuster_from_scene(scene, precision="mixed", irls="none", gps=False, constant_cameras=True)
    ba.add_absolute_pan("0", 0.1, 0.1)
    batch = pybundle.BundleBatch()
    batch.add(ba)
    with pytest.raises(Exception, match="orientation"):
        batch.run()
