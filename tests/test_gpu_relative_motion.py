"""Relative motions between rig instances and their reconstruction scales in
the GPU solve: the reference's own relative-motion tests
(opensfm/test/test_bundle.py:167-452) and a solve against the FP64 CPU
oracle.

The scales are camera-side unknowns of their own (one-coordinate blocks
after the rig cameras); the relative motions are host terms coupling two
instances and up to two scales (bundle_adjuster.cc:872-910).
"""
import numpy as np
import pytest

from oracle import oracle
from opensfm_gb300 import pybundle, pygeometry
from opensfm_gb300 import synthetic as syn
from opensfm_gb300.pybundle import adjuster_from_scene

pytestmark = pytest.mark.gpu


def _adjuster(precision, n):
    ba = pybundle.BundleAdjuster()
    ba.set_precision(precision)
    ba.set_skip_initial_reweighting(True)
    cam = pygeometry.Camera.create_perspective(1.0, 0.0, 0.0)
    ba.add_camera("cam1", cam, cam, True)
    ba.add_rig_camera("rig_cam1", pygeometry.Pose(), pygeometry.Pose(), True)
    for i in range(n):
        iid = str(i + 1)
        ba.add_rig_instance(iid, pygeometry.Pose(np.zeros(3), np.zeros(3)), {iid: "cam1"}, {iid: "rig_cam1"}, False)
    return ba


def _motion(i, j, t, observed=False):
    return pybundle.RelativeMotion(i, j, np.zeros(3), np.asarray(t, np.float64), 1, 1, observed)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("shared,expected", [(True, (0.5, 0.5)), (False, (4.0, 0.5))])
def test_pair(precision, shared, expected):
    # test_bundle.py:167-194 (shared scale) and :268-295 (one scale per
    # instance: instance 1's scale has no residual and keeps its value)
    ba = _adjuster(precision, 2)
    ba.add_reconstruction("12", False)
    ba.add_reconstruction_instance("12", 4, "1")
    ba.add_reconstruction_instance("12", 4, "2")
    ba.set_scale_sharing("12", shared)
    ba.add_relative_motion(_motion("1", "2", [-1, 0, 0]))
    ba.add_rig_instance_position_prior("1", np.zeros(3), np.ones(3), "")
    ba.add_rig_instance_position_prior("2", np.array([2.0, 0, 0]), np.ones(3), "")
    ba.run()
    assert np.allclose(ba.get_rig_instance_pose("1").translation, [0, 0, 0], atol=1e-6)
    assert np.allclose(ba.get_rig_instance_pose("2").translation, [-2, 0, 0], atol=1e-6)
    r12 = ba.get_reconstruction("12")
    assert np.allclose([r12.get_scale("1"), r12.get_scale("2")], expected)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_four_cams_single_reconstruction(precision):
    # test_bundle.py:298-362
    ba = _adjuster(precision, 4)
    ba.add_reconstruction("1234", False)
    for i in "1234":
        ba.add_reconstruction_instance("1234", 1, i)
    ba.set_scale_sharing("1234", True)
    ba.add_relative_motion(_motion("1", "2", [-1, 0, 0]))
    ba.add_relative_motion(_motion("1", "3", [0, -1, 0]))
    ba.add_relative_motion(_motion("1", "4", [0, 0, -1]))
    ba.add_rig_instance_position_prior("1", np.zeros(3), np.ones(3), "")
    ba.add_rig_instance_position_prior("2", np.array([2.0, 0, 0]), np.ones(3), "")
    ba.add_rig_instance_position_prior("3", np.array([0, 2.0, 0]), np.ones(3), "")
    ba.run()
    for i, t in zip("1234", ([0, 0, 0], [-2, 0, 0], [0, -2, 0], [0, 0, -2])):
        assert np.allclose(ba.get_rig_instance_pose(i).translation, t, atol=1e-6), (i, t)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_four_cams_double_reconstruction(precision):
    # test_bundle.py:365-452: observed scales on two of the motions
    ba = _adjuster(precision, 4)
    for rec, members in (("12", "12"), ("34", "34")):
        ba.add_reconstruction(rec, False)
        for i in members:
            ba.add_reconstruction_instance(rec, 1, i)
        ba.set_scale_sharing(rec, False)
    ba.add_relative_motion(_motion("1", "2", [-0.5, -0.5, -0.5], observed=True))
    ba.add_relative_motion(_motion("3", "2", [0.5, 0.5, 0.5]))
    ba.add_relative_motion(_motion("3", "4", [-2, -2, -2], observed=True))
    ba.add_relative_motion(_motion("2", "3", [-2, -2, -2]))
    ba.add_rig_instance_position_prior("1", np.zeros(3), np.ones(3), "")
    ba.add_rig_instance_position_prior("4", np.array([3.0, 3, 3]), np.ones(3), "")
    ba.run()
    for i, o in zip("1234", ([0, 0, 0], [1, 1, 1], [2, 2, 2], [3, 3, 3])):
        assert np.allclose(ba.get_rig_instance_pose(i).get_origin(), o, atol=1e-6), (i, o)
    r12, r34 = ba.get_reconstruction("12"), ba.get_reconstruction("34")
    assert np.allclose([r12.get_scale("1"), r12.get_scale("2")], 0.5)
    assert np.allclose([r34.get_scale("3"), r34.get_scale("4")], 2.0)


def _rot(a):
    a = np.asarray(a, np.float64)
    t = np.linalg.norm(a)
    if t < 1e-300:
        return np.eye(3)
    k = a / t
    K = np.array([[0, -k[2], k[1]], [k[2], 0, -k[0]], [-k[1], k[0], 0]])
    return np.eye(3) + np.sin(t) * K + (1 - np.cos(t)) * K @ K


def _log(M):
    th = np.arccos(np.clip((np.trace(M) - 1) / 2, -1, 1))
    return th / (2 * np.sin(th)) * np.array([M[2, 1] - M[1, 2], M[0, 2] - M[2, 0], M[1, 0] - M[0, 1]])


@pytest.mark.parametrize("solver", ["ITERATIVE_SCHUR", "SPARSE_SCHUR"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_ring_relative_motions_match_oracle(precision, solver):
    # Ring scene with GPS priors; two reconstructions (shots 0-9 and
    # 10-19), each with one shared scale starting at 1; relative motions
    # between neighbours whose translations are 0.8 x the true ones
    # (3 mrad and 1 cm noise): both scales settle near 0.8
    scene = syn.ring_scene(n_points=1500, seed=13)
    true = scene.extras["true_poses"]
    rng = np.random.default_rng(4)
    n = len(scene.shot_camera)
    scene.extras["gps"] = np.ascontiguousarray(true[:, 3:] + rng.normal(0, 0.05, (n, 3)))
    scene.extras["gps_std"] = np.full((n, 3), 0.1)
    M = np.diag([100.0, 100, 100, 10, 10, 10, 1])
    rel, motions = [], []
    for s in range(n):
        t = (s + 1) % n
        Ri, Rj = _rot(true[s][:3]), _rot(true[t][:3])
        rij = -_log(Ri.T @ Rj) + rng.normal(0, 0.003, 3)
        tij = 0.8 * Rj.T @ (true[s, 3:] - true[t, 3:]) + rng.normal(0, 0.01, 3)
        rel.append(("relative_motion", (s, t), np.r_[rij, tij, 1.0, 0.0, M.ravel(), 1.0, s >= n // 2, t >= n // 2]))
        rm = pybundle.RelativeMotion(str(s), str(t), rij, tij, 1.0, 1.0, False)
        rm.set_scale_matrix(M)
        motions.append(rm)
    ref = oracle.solve(scene, loss=("HuberLoss", 1.0), irls="none", max_iterations=100, gps=True, relative=rel,
                       scales=[(1.0, True), (1.0, True)])
    assert ref["termination"] == 1 and np.allclose(ref["scales"], 0.8, atol=2e-3)
    ba = adjuster_from_scene(scene, precision=precision, loss=("HuberLoss", 1.0), irls="none", max_iterations=100,
                             gps=True, linear_solver=solver, pcg_tolerance=1e-10 if precision == "fp64" else 1e-4)
    for rec, members in (("A", range(0, n // 2)), ("B", range(n // 2, n))):
        ba.add_reconstruction(rec, False)
        for i in members:
            ba.add_reconstruction_instance(rec, 1.0, str(i))
    for rm in motions:
        ba.add_relative_motion(rm)
    ba.run()
    s = ba.summary()
    assert s["usable"]
    assert abs(s["final_cost"] - ref["final_cost"]) / ref["final_cost"] < 1e-6, (s["final_cost"], ref["final_cost"])
    got = [ba.get_reconstruction("A").get_scale("0"), ba.get_reconstruction("B").get_scale("10")]
    np.testing.assert_allclose(got, ref["scales"], atol=1e-5 if precision == "fp64" else 1e-4)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_four_cams_one_fixed(precision):
    # test_bundle.py:455-526
    ba = pybundle.BundleAdjuster()
    ba.set_precision(precision)
    ba.set_skip_initial_reweighting(True)
    cam = pygeometry.Camera.create_perspective(1.0, 0.0, 0.0)
    ba.add_camera("cam1", cam, cam, True)
    ba.add_rig_camera("rig_cam1", pygeometry.Pose(), pygeometry.Pose(), True)
    for i in range(4):
        iid = str(i + 1)
        ba.add_rig_instance(iid, pygeometry.Pose(np.zeros(3), np.zeros(3)), {iid: "cam1"}, {iid: "rig_cam1"}, i == 0)
    ba.add_reconstruction("1234", False)
    for i in "1234":
        ba.add_reconstruction_instance("1234", 1, i)
    ba.set_scale_sharing("1234", True)
    ba.add_relative_motion(_motion("1", "2", [-1, 0, 0]))
    ba.add_relative_motion(_motion("1", "3", [0, -1, 0]))
    ba.add_relative_motion(_motion("1", "4", [0, 0, -1]))
    ba.add_rig_instance_position_prior("1", np.array([100.0, 0, 0]), np.ones(3), "")
    ba.add_rig_instance_position_prior("2", np.array([2.0, 0, 0]), np.ones(3), "")
    ba.add_rig_instance_position_prior("3", np.array([0, 2.0, 0]), np.ones(3), "")
    ba.run()
    for i, t in zip("1234", ([0, 0, 0], [-2, 0, 0], [0, -2, 0], [0, 0, -2])):
        assert np.allclose(ba.get_rig_instance_pose(i).translation, t, atol=1e-6), (i, t)
