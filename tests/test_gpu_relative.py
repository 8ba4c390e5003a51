"""Constraints between shots -- relative rotations, common positions, linear
motion -- in the GPU solve, against the FP64 CPU oracle.

They are host terms of the camera-side system (bundle_adjuster.cc:
912-999, 1080-1138) coupling two or three rig instances; the GPU solve adds
their off-diagonal Gauss-Newton blocks to the implicit Schur product and
the dense reduced camera system.  GPS priors fix the gauge (a common
position is not invariant to the scale of the scene).  Bars as in
test_gpu_solver.py.
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


def _log(M):
    th = np.arccos(np.clip((np.trace(M) - 1) / 2, -1, 1))
    return th / (2 * np.sin(th)) * np.array([M[2, 1] - M[1, 2], M[0, 2] - M[2, 0], M[1, 0] - M[0, 1]])


def _scene_and_constraints(seed=13):
    """Ring scene with GPS priors; relative rotations between neighbours
    (0.005 rad noise, 0.01 rad std), common positions of opposite shots
    (25 m horizontal margin: the heights are pulled together), linear
    motion over consecutive triples."""
    scene = syn.ring_scene(n_points=1500, seed=seed)
    true = scene.extras["true_poses"]
    rng = np.random.default_rng(4)
    n = len(scene.shot_camera)
    scene.extras["gps"] = np.ascontiguousarray(true[:, 3:] + rng.normal(0, 0.05, (n, 3)))
    scene.extras["gps_std"] = np.full((n, 3), 0.1)
    rel = []
    for s in range(n):
        t = (s + 1) % n
        rij = -_log(_rot(true[s][:3]).T @ _rot(true[t][:3])) + rng.normal(0, 0.005, 3)
        rel.append(("relative_rotation", (s, t), np.r_[rij, (np.eye(3) / 0.01).ravel()]))
    for s in range(n // 2):
        rel.append(("common_position", (s, s + n // 2), [25.0, 1.0]))
    for s in range(n):
        rel.append(("linear_motion", (s, (s + 1) % n, (s + 2) % n), [0.5, 0.1, 0.05]))
    return scene, rel


def _add(ba, rel):
    for kind, shots, prm in rel:
        sh = [str(s) for s in shots]
        if kind == "relative_rotation":
            rr = pybundle.RelativeRotation(sh[0], sh[1], prm[:3])
            rr.set_scale_matrix(np.asarray(prm[3:]).reshape(3, 3))
            ba.add_relative_rotation(rr)
        elif kind == "common_position":
            ba.add_common_position(sh[0], sh[1], prm[0], prm[1])
        else:
            ba.add_linear_motion(sh[0], sh[1], sh[2], prm[0], prm[1], prm[2])


@pytest.mark.parametrize("solver", ["ITERATIVE_SCHUR", "SPARSE_SCHUR"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_ring_relative_constraints_match_oracle(precision, solver):
    scene, rel = _scene_and_constraints()
    ref = oracle.solve(scene, loss=("HuberLoss", 1.0), irls="none", max_iterations=100, gps=True, relative=rel)
    free = oracle.solve(scene, loss=("HuberLoss", 1.0), irls="none", max_iterations=100, gps=True)
    assert ref["termination"] == 1
    assert ref["final_cost"] > free["final_cost"] * 1.0005  # the constraints pull against the images
    ba = adjuster_from_scene(scene, precision=precision, loss=("HuberLoss", 1.0), irls="none", max_iterations=100,
                             gps=True, linear_solver=solver, pcg_tolerance=1e-10 if precision == "fp64" else 1e-4)
    _add(ba, rel)
    ba.run()
    s = ba.summary()
    assert s["usable"]
    rel_err = abs(s["final_cost"] - ref["final_cost"]) / ref["final_cost"]
    assert rel_err < 1e-6, (s["final_cost"], ref["final_cost"])
    got = np.stack([ba.get_rig_instance_pose(str(i)).rotation for i in range(len(scene.shot_camera))])
    want = np.stack([pygeometry.Pose.from_ba_data(p).rotation for p in ref["instances"]])
    np.testing.assert_allclose(got, want, atol=1e-4)


@pytest.mark.parametrize("kind", ["relative_rotation", "common_position", "linear_motion"])
def test_each_kind_matches_oracle(kind):
    scene, rel = _scene_and_constraints(seed=21)
    sub = [c for c in rel if c[0] == kind]
    ref = oracle.solve(scene, loss=("HuberLoss", 1.0), irls="none", max_iterations=100, gps=True, relative=sub)
    ba = adjuster_from_scene(scene, precision="fp64", loss=("HuberLoss", 1.0), irls="none", max_iterations=100,
                             gps=True, linear_solver="SPARSE_SCHUR")
    _add(ba, sub)
    ba.run()
    s = ba.summary()
    assert abs(s["final_cost"] - ref["final_cost"]) / ref["final_cost"] < 1e-6, (s["final_cost"], ref["final_cost"])


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_ring_relative_irls_and_loss_match_oracle(precision):
    # groups ROT (20), POS (10), MOTION (20) are reweighted; the relative
    # rotations under SoftLOneLoss(2)
    scene, rel = _scene_and_constraints()
    ref = oracle.solve(scene, irls="mixture", max_iterations=100, gps=True, relative=rel,
                       relative_loss=("SoftLOneLoss", 2.0))
    ba = adjuster_from_scene(scene, precision=precision, irls="mixture", max_iterations=100, gps=True,
                             linear_solver="SPARSE_SCHUR")
    ba.set_relative_motion_loss_function("SoftLOneLoss", 2.0)
    _add(ba, rel)
    ba.run()
    s = ba.summary()
    assert s["usable"]
    rel_err = abs(s["final_cost"] - ref["final_cost"]) / ref["final_cost"]
    assert rel_err < (1e-6 if precision == "fp64" else 1e-5), (s["final_cost"], ref["final_cost"])


def test_unknown_relative_loss_fails_the_run():
    scene, rel = _scene_and_constraints()
    ba = adjuster_from_scene(scene, precision="fp64", irls="none", gps=True)
    ba.set_relative_motion_loss_function("NoSuchLoss", 1.0)
    _add(ba, rel[:1])
    with pytest.raises(RuntimeError, match="NoSuchLoss"):
        ba.run()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_gauge_fix_matches_oracle(precision):
    # no GPS: the origin shot's instance is held and the distance to the
    # scale shot's instance kept, which fixes all seven gauge freedoms
    scene = syn.ring_scene(n_points=1500, seed=17)
    ref = oracle.solve(scene, loss=("HuberLoss", 1.0), irls="none", max_iterations=100, gps=False, gauge=(0, 10))
    assert ref["termination"] == 1
    ba = adjuster_from_scene(scene, precision=precision, loss=("HuberLoss", 1.0), irls="none", max_iterations=100,
                             gps=False, linear_solver="SPARSE_SCHUR")
    ba.set_gauge_fix_shots("0", "10")
    ba.run()
    s = ba.summary()
    assert s["usable"]
    assert abs(s["final_cost"] - ref["final_cost"]) / ref["final_cost"] < 1e-6, (s["final_cost"], ref["final_cost"])
    p0 = ba.get_rig_instance_pose("0")
    np.testing.assert_allclose(p0.rotation, pygeometry.Pose.from_ba_data(scene.rig_instance_poses[0]).rotation,
                               atol=1e-12)
    # the scale is held by a weak term (log of the distance ratio, unit
    # weight): the run stops on the function tolerance with the ratio a
    # little off 1, where the oracle stops too.  Along this nearly flat
    # direction the mixed solve's end point moves by ~1e-4 between runs
    # (FP32 atomics' summation order).
    d0 = np.linalg.norm(scene.rig_instance_poses[0, 3:] - scene.rig_instance_poses[10, 3:])
    d1 = np.linalg.norm(ba.get_rig_instance_pose("0").get_origin() - ba.get_rig_instance_pose("10").get_origin())
    d_ref = np.linalg.norm(ref["instances"][0, 3:] - ref["instances"][10, 3:])
    exact = precision == "fp64"
    assert abs(d1 / d0 - 1) < 5e-3 and abs(d1 / d_ref - 1) < (1e-5 if exact else 1e-3), (d0, d1, d_ref)
    # the gauge is fixed: the same points as the oracle
    np.testing.assert_allclose(ba.get_points(), ref["points"], atol=1e-4 if exact else 2e-2)


def _bell(size, r, mu_x, mu_y):
    # the cost surface of test_bundle.py:675-693: 1 - a normalised Gaussian
    x, y = np.meshgrid(np.linspace(-r, r, size), np.linspace(r, -r, size))
    z = np.exp(-((x - mu_x) ** 2 / (2 * (r / 2) ** 2) + (y - mu_y) ** 2 / (2 * (r / 2) ** 2)))
    return 1 - z / z.max()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_heatmap_singletons(precision):
    # test_bundle.py:650-735 without the reconstruction bookkeeping (its
    # scales enter only relative motions): three shots pulled to the bell's
    # minimum shifted by their offsets
    ba = pybundle.BundleAdjuster()
    ba.set_precision(precision)
    ba.set_skip_initial_reweighting(True)
    cam = pygeometry.Camera.create_perspective(1.0, 0.0, 0.0)
    ba.add_camera("cam1", cam, cam, True)
    ba.add_rig_camera("rig_cam1", pygeometry.Pose(), pygeometry.Pose(), True)
    for i in range(3):
        ba.add_rig_instance(str(i + 1), pygeometry.Pose(np.zeros(3), np.zeros(3)), {str(i + 1): "cam1"},
                            {str(i + 1): "rig_cam1"}, False)
    hmap_x, hmap_y, size, rad = 1, -1, 101, 10
    res = 2 * rad / (size - 1)
    ba.add_heatmap("hmap1", _bell(size, rad, hmap_x, hmap_y).flatten().tolist(), size, res)
    offsets = [(2, 0), (0, 2), (-2, 0)]
    for i, (xo, yo) in enumerate(offsets):
        ba.add_absolute_position_heatmap(str(i + 1), "hmap1", xo, yo, 1.0)
    ba.run()
    for i, (xo, yo) in enumerate(offsets):
        s = ba.get_rig_instance_pose(str(i + 1))
        assert np.allclose(-s.translation, [xo + hmap_x, yo + hmap_y, 0], atol=res), s.translation


@pytest.mark.parametrize("solver", ["ITERATIVE_SCHUR", "SPARSE_SCHUR"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_ring_heatmap_matches_oracle(precision, solver):
    # every shot looked up in one 30 m bell grid, offset so that its minimum
    # sits 1.2 m from the shot's true horizontal position (std 2 mm: the
    # pull is felt); GPS priors hold the height
    scene, _ = _scene_and_constraints(seed=23)
    true = scene.extras["true_poses"]
    size, rad = 121, 15.0
    res = 2 * rad / (size - 1)
    grid = _bell(size, rad, 0.0, 0.0)
    rel = [("heatmap", (s,), [true[s, 3] + 1.0, true[s, 4] - 0.7, 0.002]) for s in range(len(scene.shot_camera))]
    ref = oracle.solve(scene, loss=("HuberLoss", 1.0), irls="none", max_iterations=100, gps=True, relative=rel,
                       heatmap=(grid, size, res))
    free = oracle.solve(scene, loss=("HuberLoss", 1.0), irls="none", max_iterations=100, gps=True)
    assert ref["termination"] == 1 and ref["final_cost"] > free["final_cost"] * 1.001
    ba = adjuster_from_scene(scene, precision=precision, loss=("HuberLoss", 1.0), irls="none", max_iterations=100,
                             gps=True, linear_solver=solver, pcg_tolerance=1e-10 if precision == "fp64" else 1e-4)
    ba.add_heatmap("bell", grid.ravel(), size, res)
    for _, (s,), (xo, yo, std) in rel:
        ba.add_absolute_position_heatmap(str(s), "bell", xo, yo, std)
    ba.run()
    s = ba.summary()
    assert s["usable"]
    assert abs(s["final_cost"] - ref["final_cost"]) / ref["final_cost"] < 1e-6, (s["final_cost"], ref["final_cost"])


def _three(precision, fixed=(False, False, False), rotations=((0, 0, 0),) * 3):
    ba = pybundle.BundleAdjuster()
    ba.set_precision(precision)
    ba.set_skip_initial_reweighting(True)
    cam = pygeometry.Camera.create_perspective(1.0, 0.0, 0.0)
    ba.add_camera("cam1", cam, cam, True)
    ba.add_rig_camera("rig_cam1", pygeometry.Pose(), pygeometry.Pose(), True)
    for i in range(3):
        iid = str(i + 1)
        ba.add_rig_instance(iid, pygeometry.Pose(np.array(rotations[i], np.float64), np.zeros(3)), {iid: "cam1"},
                            {iid: "rig_cam1"}, fixed[i])
    return ba


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_linear_motion_prior_position(precision):
    # test_bundle.py:529-552
    ba = _three(precision)
    ba.add_rig_instance_position_prior("1", np.zeros(3), np.ones(3), "")
    ba.add_rig_instance_position_prior("3", np.array([2.0, 0, 0]), np.ones(3), "")
    ba.add_linear_motion("1", "2", "3", 0.5, 0.1, 0.1)
    ba.run()
    for i, t in zip("123", ([0, 0, 0], [-1, 0, 0], [-2, 0, 0])):
        assert np.allclose(ba.get_rig_instance_pose(i).translation, t, atol=1e-6), (i, t)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_linear_motion_prior_rotation(precision):
    # test_bundle.py:555-590
    ba = _three(precision, fixed=(True, False, True), rotations=((0, 0, 0), (0, 0, 0), (0, 1, 0)))
    ba.add_linear_motion("1", "2", "3", 0.3, 0.1, 0.1)
    ba.run()
    assert np.allclose(ba.get_rig_instance_pose("2").rotation, [0, 0.3, 0], atol=1e-6)
