"""Local bundles driven through the GPU adjuster (ba_helpers.cc:437-720
BundleLocal, set up by opensfm_gb300.ba_helpers): one local bundle, and
several at once through the batched solver.  The interior moves, the
boundary is held, and every solve lowers its cost."""
import numpy as np
import pytest

from opensfm_gb300 import ba_helpers
from opensfm_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu


def _scene():
    return syn.street_scene(n_shots=40, n_points=3000, seed=11, outlier_ratio=0.0)


def test_bundle_local_moves_the_interior_only():
    scene = _scene()
    poses, points, lp = ba_helpers.bundle_local(scene, 20, max_shots=10, use_gps=False, loss=("SoftLOneLoss", 1.0))
    s = lp.adjuster.summary()
    assert s["usable"] and s["final_cost"] < s["initial_cost"]
    free = set(lp.free_instances)
    assert free and len(lp.boundary) > 0
    moved = np.abs(poses - scene.rig_instance_poses).max(axis=1) > 0
    assert set(np.nonzero(moved)[0].tolist()) <= free
    assert moved[sorted(free)].any()
    # only points seen from the interior change
    changed = np.abs(points - scene.points).max(axis=1) > 0
    assert set(np.nonzero(changed)[0].tolist()) <= set(lp.point_ids.tolist())


def test_bundle_local_batch_solves_every_problem():
    scene = _scene()
    poses, points, problems = ba_helpers.bundle_local_batch(scene, [5, 20, 35], max_shots=8, use_gps=False,
                                                            loss=("SoftLOneLoss", 1.0))
    assert len(problems) == 3
    for lp in problems:
        s = lp.adjuster.summary()
        assert s["usable"] and s["final_cost"] <= s["initial_cost"], s
    assert np.isfinite(poses).all() and np.isfinite(points).all()


def test_bundle_stochastic_rounds_lower_the_cost():
    # BundleStochastic (ba_helpers.cc:1231-1370): three rounds of local
    # bundles around random seeds, each from the previous round's result
    scene = _scene()
    poses, points, report = ba_helpers.bundle_stochastic(scene, max_shots=10, random_shots=3, max_rounds=3,
                                                         use_gps=False, loss=("SoftLOneLoss", 1.0))
    assert report["num_rounds"] == 3 and len(report["rounds"]) == 3
    for r in report["rounds"]:
        s = r["summary"]
        assert s["usable"] and s["final_cost"] <= s["initial_cost"], s
        assert 3 <= r["interior"] <= 12
    assert np.isfinite(poses).all() and np.isfinite(points).all()


def test_bundle_shot_poses_refines_the_given_shots():
    # BundleShotPoses: two shots moved off, refined against constant points
    scene = _scene()
    moved = np.array(scene.rig_instance_poses, copy=True)
    moved[[5, 6], 3:] += 0.3
    scene.rig_instance_poses = moved
    poses, lp = ba_helpers.bundle_shot_poses(scene, [5, 6], use_gps=False, loss=("SoftLOneLoss", 1.0))
    s = lp.adjuster.summary()
    assert s["usable"] and s["final_cost"] < 0.5 * s["initial_cost"], s
    others = np.setdiff1d(np.arange(len(poses)), [5, 6])
    np.testing.assert_array_equal(poses[others], moved[others])
    assert np.abs(poses[[5, 6]] - moved[[5, 6]]).max() > 0.01
