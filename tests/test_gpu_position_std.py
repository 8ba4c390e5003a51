"""Adjusted GPS standard deviations in the GPU solve against the FP64 CPU
oracle: set_adjust_absolute_position_std turns every GPS prior into a host
term divided by its scale group's std multiplier and adds the multiplier's
StdDeviationConstraint (bundle_adjuster.cc:772-838); the oracle solves the
same problem written as explicit relative terms."""
import numpy as np
import pytest

from oracle import oracle
from opensfm_gb300 import pybundle, pygeometry
from opensfm_gb300 import synthetic as syn
from opensfm_gb300.pybundle import adjuster_from_scene

pytestmark = pytest.mark.gpu


def _scene(noise):
    scene = syn.ring_scene(n_points=1500, seed=5)
    true = scene.extras["true_poses"]
    n = len(scene.shot_camera)
    rng = np.random.default_rng(8)
    scene.extras["gps"] = np.ascontiguousarray(true[:, 3:] + rng.normal(0, noise, (n, 3)))
    scene.extras["gps_std"] = np.full((n, 3), 0.1)
    return scene


@pytest.mark.parametrize("solver", ["ITERATIVE_SCHUR", "DENSE_SCHUR"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_adjusted_gps_matches_oracle(precision, solver):
    scene = _scene(0.3)
    gps, std = scene.extras["gps"], scene.extras["gps_std"]
    rel = [("gps_std", (s,), np.r_[gps[s], std[s], 0.0]) for s in range(len(gps))]
    rel.append(("std_deviation", (), [0.0]))
    ref = oracle.solve(scene, loss=("HuberLoss", 1.0), irls="none", max_iterations=200, gps=False, relative=rel,
                       scales=[(1.0, True)])
    assert ref["termination"] == 1 and ref["scales"][0] > 1.0
    ba = adjuster_from_scene(scene, precision=precision, loss=("HuberLoss", 1.0), irls="none", max_iterations=200,
                             gps=True, linear_solver=solver, pcg_tolerance=1e-10 if precision == "fp64" else 1e-4)
    ba.set_adjust_absolute_position_std(True)
    ba.run()
    s = ba.summary()
    assert s["usable"]
    assert abs(s["final_cost"] - ref["final_cost"]) / ref["final_cost"] < 1e-6, (s["final_cost"], ref["final_cost"])
    tol = 1e-4 if precision == "fp64" else 1e-3
    for i, p in enumerate(ref["instances"]):
        got = ba.get_rig_instance_pose(str(i)).translation
        np.testing.assert_allclose(got, pygeometry.Pose.from_ba_data(p).translation, atol=tol)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_adjusting_lowers_the_cost_of_noisy_gps(precision):
    # with the multiplier free the GPS priors' weight drops, and the
    # multiplier itself is removed again after the run (a second run
    # without adjusting solves the plain problem)
    scene = _scene(0.3)
    plain = adjuster_from_scene(scene, precision=precision, irls="none", max_iterations=100)
    plain.run()
    adj = adjuster_from_scene(scene, precision=precision, irls="none", max_iterations=100)
    adj.set_adjust_absolute_position_std(True)
    adj.run()
    assert adj.summary()["final_cost"] < plain.summary()["final_cost"]
    adj.set_adjust_absolute_position_std(False)
    adj.run()
    rel = abs(adj.summary()["final_cost"] - plain.summary()["final_cost"]) / plain.summary()["final_cost"]
    assert rel < 1e-3


def test_batch_rejects_adjusted_gps_and_restores_the_priors():
    # the batch set-up fails on the multiplier (a free camera-side block)
    # and leaves the adjuster as it was: a plain run afterwards still sees
    # its GPS priors
    scene = _scene(0.3)
    ba = adjuster_from_scene(scene, precision="mixed", irls="none", constant_cameras=True)
    ba.set_adjust_absolute_position_std(True)
    batch = pybundle.BundleBatch()
    batch.add(ba)
    with pytest.raises(Exception, match="batched solves"):
        batch.run()
    ba.set_adjust_absolute_position_std(False)
    ba.run()
    ref = adjuster_from_scene(scene, precision="mixed", irls="none", constant_cameras=True)
    ref.run()
    rel = abs(ba.summary()["final_cost"] - ref.summary()["final_cost"]) / ref.summary()["final_cost"]
    assert rel < 1e-5
