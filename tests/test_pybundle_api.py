"""API semantics of the BundleAdjuster drop-in (host code only, no GPU).

Mirrors the reference's error conventions (bundle_adjuster.cc: unknown
camera / rig / point ids raise std::runtime_error -> RuntimeError; an unknown
shot or point in add_point_projection_observation raises std::out_of_range ->
IndexError) and the toy-scene getters of
bundle/test/bundle_adjuster_api_test.cc:43-305.
"""
import numpy as np
import pytest

from opensfm_gb300 import pybundle, pygeometry


@pytest.fixture()
def ba():
    b = pybundle.BundleAdjuster()
    b.set_skip_initial_reweighting(True)
    cam = pygeometry.Camera.create_perspective(1.0, 0.0, 0.0)
    b.add_camera("cam1", cam, cam, True)
    b.add_rig_camera("rig_cam1", pygeometry.Pose(), pygeometry.Pose(), True)
    return b


def test_unicode_and_byte_ids():
    # test_bundle.py:20-34
    b = pybundle.BundleAdjuster()
    cam = pygeometry.Camera.create_perspective(0.4, 0.1, -0.01)
    b.add_camera("A\xb2", cam, cam, True)
    b.add_camera(b"A_2", cam, cam, True)
    assert b.get_camera("A\xb2").focal == pytest.approx(0.4)
    assert b.get_camera(b"A_2").k1 == pytest.approx(0.1)


def test_unknown_ids_raise(ba):
    with pytest.raises(RuntimeError):
        ba.add_rig_instance("1", pygeometry.Pose(), {"s1": "nope"}, {"s1": "rig_cam1"}, False)
    with pytest.raises(RuntimeError):
        ba.add_rig_instance("1", pygeometry.Pose(), {"s1": "cam1"}, {"s1": "nope"}, False)
    with pytest.raises(RuntimeError):
        ba.add_rig_instance_position_prior("missing", [0, 0, 0], [1, 1, 1], "")
    with pytest.raises(RuntimeError):
        ba.add_point_prior("missing", [0, 0, 0], [1, 1, 1], True)
    with pytest.raises(RuntimeError):
        ba.get_camera("missing")
    with pytest.raises(RuntimeError):
        ba.get_point("missing")
    with pytest.raises(RuntimeError):
        ba.get_rig_instance_pose("missing")
    with pytest.raises(RuntimeError):
        ba.get_rig_camera_pose("missing")
    with pytest.raises(RuntimeError):
        ba.add_rig_camera("rig_cam1", pygeometry.Pose(), pygeometry.Pose(), True)  # already exists


def test_unknown_shot_or_point_in_observation_is_index_error(ba):
    ba.add_rig_instance("1", pygeometry.Pose(), {"s1": "cam1"}, {"s1": "rig_cam1"}, False)
    ba.add_point("p1", [0, 0, 1], False)
    with pytest.raises(IndexError):
        ba.add_point_projection_observation("nope", "p1", [0, 0], 1.0)
    with pytest.raises(IndexError):
        ba.add_point_projection_observation("s1", "nope", [0, 0], 1.0)
    ba.add_point_projection_observation("s1", "p1", [0, 0], 1.0)


def test_unknown_loss_and_solver_names(ba):
    with pytest.raises(RuntimeError):
        ba.set_point_projection_loss_function("NoSuchLoss", 1.0)
    for name in ("TrivialLoss", "HuberLoss", "SoftLOneLoss", "CauchyLoss", "ArctanLoss"):
        ba.set_point_projection_loss_function(name, 1.0)
    ba.set_linear_solver_type("NOT_A_SOLVER")
    with pytest.raises(RuntimeError):
        ba.run()  # validated at run time, like the reference (bundle_adjuster.cc:1161-1165)


def test_getters_round_trip(ba):
    pose = pygeometry.Pose(np.array([0.1, -0.2, 0.3]), np.array([1.0, 2.0, 3.0]))
    ba.add_rig_instance("1", pose, {"s1": "cam1"}, {"s1": "rig_cam1"}, False)
    got = ba.get_rig_instance_pose("1")
    np.testing.assert_allclose(got.rotation, pose.rotation, atol=1e-12)
    np.testing.assert_allclose(got.translation, pose.translation, atol=1e-12)
    ba.add_point("p", [1.5, -2.0, 7.0], False)
    assert ba.has_point("p") and not ba.has_point("q")
    np.testing.assert_allclose(ba.get_point("p").p, [1.5, -2.0, 7.0])
    assert ba.get_point("p").id == "p"
    cam = ba.get_camera("cam1")
    assert cam.projection_type == "perspective"
    np.testing.assert_allclose(cam.get_parameters_values(), [0.0, 0.0, 1.0])


def test_density_ratio_settings(ba):
    # bundle_adjuster.cc:464-483
    assert ba.get_default_density_ratio() == pytest.approx(1e-3)
    ba.set_default_density_ratio(0.05)
    assert ba.get_group_density_ratio("PROJ_x") == pytest.approx(0.05)
    ba.set_group_density_ratio("GPS", 1e-5)
    assert ba.get_group_density_ratio("GPS") == pytest.approx(1e-5)


def test_unsupported_constraints_raise(ba):
    ba.add_rig_instance("1", pygeometry.Pose(), {"s1": "cam1"}, {"s1": "rig_cam1"}, False)
    ba.add_point("p", np.zeros(3), False)
    # the gauge fix looks the origin shot up at once (bundle_adjuster.cc:391)
    with pytest.raises(IndexError):
        ba.set_gauge_fix_shots("a", "b")


def test_reconstruction_bookkeeping(ba):
    # bundle_adjuster.cc:219-244, 1344-1350: unknown reconstruction ids are
    # ignored by the adders and raise in get_reconstruction
    ba.add_rig_instance("1", pygeometry.Pose(), {"s1": "cam1"}, {"s1": "rig_cam1"}, False)
    ba.add_rig_instance("2", pygeometry.Pose(), {"s2": "cam1"}, {"s2": "rig_cam1"}, False)
    ba.add_reconstruction("12", False)
    ba.add_reconstruction_instance("12", 4.0, "2")
    ba.add_reconstruction_instance("12", 3.0, "1")
    ba.add_reconstruction_instance("nope", 1.0, "1")
    ba.set_scale_sharing("nope", False)
    r = ba.get_reconstruction("12")
    # shared (the default): the first instance in id order
    assert r.get_scale("2") == 3.0 and r.get_scale("1") == 3.0
    ba.set_scale_sharing("12", False)
    assert r.get_scale("2") == 4.0 and r.get_scale("1") == 3.0
    with pytest.raises(RuntimeError):
        ba.get_reconstruction("nope")
    with pytest.raises(IndexError):
        r.get_scale("3")
    ba.add_relative_motion(pybundle.RelativeMotion("1", "2", [0, 0, 0], [-1, 0, 0], 1, 1, False))


def test_relative_constraints_on_unknown_shots_are_index_errors(ba):
    ba.add_rig_instance("1", pygeometry.Pose(), {"s1": "cam1"}, {"s1": "rig_cam1"}, False)
    ba.add_rig_instance("2", pygeometry.Pose(), {"s2": "cam1"}, {"s2": "rig_cam1"}, False)
    rr = pybundle.RelativeRotation("s1", "s2", [0.1, 0.0, 0.0])
    rr.set_scale_matrix(2 * np.eye(3))
    ba.add_relative_rotation(rr)
    ba.add_common_position("s1", "s2", 0.5, 1.0)
    ba.add_linear_motion("s1", "s2", "s1", 0.5, 1.0, 1.0)
    ba.set_relative_motion_loss_function("HuberLoss", 1.0)
    with pytest.raises(IndexError):
        ba.add_relative_rotation(pybundle.RelativeRotation("s1", "nope", [0, 0, 0]))
    with pytest.raises(IndexError):
        ba.add_common_position("nope", "s2", 0.5, 1.0)
    with pytest.raises(IndexError):
        ba.add_linear_motion("s1", "s2", "nope", 0.5, 1.0, 1.0)


def test_orientation_constraint_on_unknown_shot_is_index_error(ba):
    # the reference looks the shot up with shots_.at() when Run adds the
    # block (bundle_adjuster.cc:1013-1082); here the lookup is at add time
    with pytest.raises(IndexError):
        ba.add_absolute_up_vector("1", np.array([0, -1, 0]), 1)
    ba.add_rig_instance("1", pygeometry.Pose(), {"s1": "cam1"}, {"s1": "rig_cam1"}, False)
    ba.add_absolute_up_vector("s1", np.array([0, -1, 0]), 1)
    ba.add_absolute_pan("s1", 0.1, 1)
    ba.add_absolute_tilt("s1", 0.1, 1)
    ba.add_absolute_roll("s1", 0.1, 1)
    with pytest.raises(IndexError):
        ba.add_absolute_roll("s2", 0.1, 1)


def test_camera_factories_parameter_order():
    pp = np.array([0.1, -0.05])
    c = pygeometry.Camera.create_brown(0.4, 0.9, pp, [-0.1, 0.03, 0.001, 0.001, 0.002])
    np.testing.assert_allclose(c.get_parameters_values(), [-0.1, 0.03, 0.001, 0.001, 0.002, 0.4, 0.9, 0.1, -0.05])
    assert c.focal == pytest.approx(0.4) and c.aspect_ratio == pytest.approx(0.9)
    c = pygeometry.Camera.create_dual(0.5, 0.4, -0.1, 0.01)
    np.testing.assert_allclose(c.get_parameters_values(), [0.5, -0.1, 0.01, 0.4])
    with pytest.raises(RuntimeError):
        pygeometry.Camera.create_brown(0.4, 1.0, pp, [0.1])


def test_pose_data_round_trip():
    p = pygeometry.Pose(np.array([0.3, 0.2, -0.1]), np.array([0.5, -1.0, 2.0]))
    q = pygeometry.Pose.from_ba_data(p.ba_data())
    np.testing.assert_allclose(q.rotation, p.rotation, atol=1e-14)
    np.testing.assert_allclose(q.translation, p.translation, atol=1e-14)
    np.testing.assert_allclose(p.transform_inverse(p.transform([1, 2, 3])), [1, 2, 3], atol=1e-12)


def test_run_checks_relative_constraints_before_the_solve(ba):
    # both failures come from the run's set-up, before any device work: a
    # relative motion needs its instances in a reconstruction
    # (reconstructions_assignments_.at, bundle_adjuster.cc:892-897), and the
    # relative-motion loss name must exist (CreateLossFunction, :485-499)
    ba.add_rig_instance("1", pygeometry.Pose(), {"s1": "cam1"}, {"s1": "rig_cam1"}, False)
    ba.add_rig_instance("2", pygeometry.Pose(), {"s2": "cam1"}, {"s2": "rig_cam1"}, False)
    ba.add_relative_motion(pybundle.RelativeMotion("1", "2", [0, 0, 0], [-1, 0, 0], 1, 1, False))
    with pytest.raises(IndexError):
        ba.run()
    ba.add_reconstruction("12", False)
    ba.add_reconstruction_instance("12", 1.0, "1")
    ba.add_reconstruction_instance("12", 1.0, "2")
    ba.set_relative_motion_loss_function("NoSuchLoss", 1.0)
    with pytest.raises(RuntimeError, match="NoSuchLoss"):
        ba.run()


def test_heatmap_and_residual_argument_checks(ba):
    ba.add_rig_instance("1", pygeometry.Pose(), {"s1": "cam1"}, {"s1": "rig_cam1"}, False)
    # a grid must hold a positive multiple of its width
    with pytest.raises(pybundle._lib.GbbaError):
        ba.add_heatmap("h", [0.0] * 5, 2, 1.0)
    with pytest.raises(pybundle._lib.GbbaError):
        ba.add_heatmap("h", [0.0] * 4, 0, 1.0)
    ba.add_heatmap("h", [0.0] * 4, 2, 1.0)
    with pytest.raises(IndexError):
        ba.add_absolute_position_heatmap("s1", "missing", 0.0, 0.0, 1.0)
    with pytest.raises(IndexError):
        ba.add_absolute_position_heatmap("s2", "h", 0.0, 0.0, 1.0)
    ba.add_absolute_position_heatmap("s1", "h", 0.0, 0.0, 1.0)
    # residual helpers: unknown kinds and non-positive deviations
    with pytest.raises(KeyError):
        pybundle.relative_residual("heatmap", np.zeros((2, 6)), [0.0])
    with pytest.raises(pybundle._lib.GbbaError):
        pybundle.heatmap_residual(np.zeros(6), 4, 1.0, 0.0, 0.0, 1.0, np.zeros(6))
    r, J = pybundle.heatmap_residual(np.ones(6), 3, 1.0, 0.0, 0.0, 0.5, np.zeros(6))
    assert r == pytest.approx(2.0) and np.all(J == 0.0)  # a constant grid: value / std, no slope


def test_batch_linear_solver_names():
    from opensfm_gb300.pybundle import BundleBatch
    batch = BundleBatch()
    for name in ("DENSE_SCHUR", "SPARSE_SCHUR", "ITERATIVE_SCHUR", "CGNR"):
        batch.set_linear_solver_type(name)
    with pytest.raises(Exception, match="doesn't exist"):
        batch.set_linear_solver_type("CHOLMOD")
