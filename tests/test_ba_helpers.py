"""Local-bundle helpers on the host (no GPU): the neighbourhood selection of
sfm::BAHelpers::ShotNeighborhood / DirectShotNeighbors
(opensfm/src/lib/sfm/src/ba_helpers.cc:64-136) on hand-built
co-visibility, and the set-up of the local problem (ba_helpers.cc:176-330).
"""
import numpy as np

from opensfm_gb300 import ba_helpers, scene as sc


def _chain(n_shots=6, window=25, step=10, instances=None):
    """Shot i sees points 10 i .. 10 i + 24: neighbours share 15 points,
    shots two apart 5, three apart none."""
    obs_shot, obs_point = [], []
    for i in range(n_shots):
        for p in range(step * i, step * i + window):
            obs_shot.append(i)
            obs_point.append(p)
    n_points = step * (n_shots - 1) + window
    inst = np.arange(n_shots) if instances is None else np.asarray(instances)
    n_inst = int(inst.max()) + 1
    return sc.SceneArrays(
        camera_projection=[sc.PERSPECTIVE], camera_values=np.array([[0.85, 0.0, 0.0]]),
        rig_instance_poses=np.zeros((n_inst, 6)), shot_rig_instance=inst, shot_camera=np.zeros(n_shots),
        points=np.zeros((n_points, 3)), obs_shot=np.array(obs_shot, np.int32),
        obs_point=np.array(obs_point, np.int32), obs_xy=np.zeros((len(obs_shot), 2)),
        obs_std=np.full(len(obs_shot), 1e-3))


def test_neighborhood_grows_by_shared_points():
    cov = ba_helpers.Covisibility.of(_chain())
    # radius 3: two hops of >= 10 shared points from shot 2, then every
    # shot sharing a point is boundary
    interior, boundary = ba_helpers.shot_neighborhood(cov, [2], radius=3, min_common_points=10, max_interior_size=30)
    assert interior == {0, 1, 2, 3, 4} and boundary == {5}
    # the interior budget stops the growth after one hop
    interior, boundary = ba_helpers.shot_neighborhood(cov, [2], radius=3, min_common_points=10, max_interior_size=3)
    assert interior == {1, 2, 3} and boundary == {0, 4, 5}
    # radius 1: the central shot alone
    interior, boundary = ba_helpers.shot_neighborhood(cov, [2], radius=1, min_common_points=10, max_interior_size=30)
    assert interior == {2} and boundary == {0, 1, 3, 4}
    # a high threshold admits no neighbour
    interior, boundary = ba_helpers.shot_neighborhood(cov, [2], radius=3, min_common_points=16, max_interior_size=30)
    assert interior == {2} and boundary == {0, 1, 3, 4}


def test_direct_neighbors_most_shared_first():
    cov = ba_helpers.Covisibility.of(_chain())
    # from {2}: shots 1 and 3 share 15, shots 0 and 4 share 5; a budget of
    # one takes the first of the two tied 15s (lowest index)
    assert ba_helpers.direct_shot_neighbors(cov, {2}, 1, 1) == {1}
    assert ba_helpers.direct_shot_neighbors(cov, {2}, 1, 3) == {0, 1, 3}
    assert ba_helpers.direct_shot_neighbors(cov, {2}, 6, 10) == {1, 3}


def test_rig_instance_siblings_come_along():
    # shots 2 and 3 form one rig instance: seeding from 2 brings 3, and a
    # neighbour pulls in its whole instance
    cov = ba_helpers.Covisibility.of(_chain(instances=[0, 1, 2, 2, 3, 4]))
    interior, boundary = ba_helpers.shot_neighborhood(cov, [2], radius=1, min_common_points=10, max_interior_size=30)
    assert interior == {2, 3} and boundary == {0, 1, 4, 5}
    assert ba_helpers.direct_shot_neighbors(cov, {1}, 10, 10) == {0, 2, 3}


def test_local_problem_set_up():
    scene = _chain()
    lp = ba_helpers.local_problem(scene, [2], radius=2, min_common_points=10, max_shots=30)
    assert lp.interior == {1, 2, 3} and lp.boundary == {0, 4, 5}
    # the points of the interior (10 .. 54) with all their observations;
    # boundary instances fixed
    np.testing.assert_array_equal(lp.point_ids, np.arange(10, 55))
    L, h = lp.adjuster._L, lp.adjuster._h
    assert int(L.gbba_num_points(h)) == 45
    keep = np.isin(scene.obs_point, np.arange(10, 55))
    assert int(L.gbba_num_projections(h)) == int(keep.sum())
    assert sorted(lp.free_instances) == [1, 2, 3] and not lp.has_position_priors
