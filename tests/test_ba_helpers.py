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


def test_select_tracks_grid_keeps_the_longest_track_per_cell():
    # SelectTracksGrid (ba_helpers.cc:938-1004) on a 2 x 2 grid of a 100 x 100
    # image.  Track lengths: p1 3, p2 2, p5 2, the others 1.  Shot 0 keeps
    # p1 (over p0) in cell 0, p2 in cell 1 and p3 in cell 3; shot 1 skips
    # the already selected p1 and keeps p4 (cell 2) and p5 (cell 0, out of
    # the image: clamped)
    obs = [(0, 0, (-0.3, -0.3)), (0, 1, (-0.2, -0.2)), (0, 2, (0.3, -0.3)), (0, 3, (0.3, 0.3)),
           (1, 1, (-0.3, 0.3)), (1, 4, (-0.2, 0.2)), (1, 5, (-0.9, -0.9)),
           (2, 1, (0.0, 0.0)), (2, 2, (0.0, 0.0)), (2, 5, (0.0, 0.0))]
    scene = sc.SceneArrays(
        camera_projection=[sc.PERSPECTIVE], camera_values=np.array([[0.0, 0.0, 1.0]]),
        rig_instance_poses=np.zeros((3, 6)), shot_rig_instance=np.arange(3), shot_camera=np.zeros(3),
        points=np.zeros((6, 3)), obs_shot=np.array([o[0] for o in obs], np.int32),
        obs_point=np.array([o[1] for o in obs], np.int32), obs_xy=np.array([o[2] for o in obs], np.float64),
        obs_std=np.full(len(obs), 1e-3))
    cov = ba_helpers.Covisibility.of(scene)
    selected, other = ba_helpers.select_tracks_grid(scene, cov, {0, 1}, 2, 100, 100)
    assert selected.tolist() == [1, 2, 3, 4, 5] and other.tolist() == [0]
    # one cell per image: the longest track of each shot
    selected, other = ba_helpers.select_tracks_grid(scene, cov, {0, 1}, 1, 100, 100)
    assert selected.size == 0 and other.size == 0  # grid_size <= 1 selects nothing
    selected, _ = ba_helpers.select_tracks_grid(scene, cov, {0}, 2, 100, 100)
    assert selected.tolist() == [1, 2, 3]
    # the local problem takes the grid selection when the image size is known
    lp = ba_helpers.local_problem(scene, [0], radius=1, min_common_points=1, grid_size=2, image_size=(100, 100))
    assert lp.point_ids.tolist() == [1, 2, 3] and lp.other_tracks.tolist() == [0]


def test_stochastic_rounds_and_seeds():
    # BundleStochastic (ba_helpers.cc:1246-1266): K = ceil(3 S / N) rounds,
    # capped, N = min(max shots, S)
    assert ba_helpers.stochastic_rounds(4000, 500, 100) == (24, 500)
    assert ba_helpers.stochastic_rounds(4000, 50, 100) == (100, 50)
    assert ba_helpers.stochastic_rounds(10, 500, 100) == (3, 10)
    assert ba_helpers.stochastic_rounds(0, 500, 100) == (1, 1)
    # seeds: distinct within a round, drawn by a partial shuffle carried
    # over rounds
    rng = np.random.default_rng(42)
    ids = list(range(30))
    first = ba_helpers.stochastic_seeds(rng, ids, 20)
    assert len(set(first)) == 20 and sorted(ids) == list(range(30))
    assert ids[:20] == first
    assert len(ba_helpers.stochastic_seeds(rng, ids, 100)) == 30


def test_shot_poses_problem_set_up():
    # BundleShotPoses: the given shots' observations only, every point they
    # see held constant; shot 3 shares its rig instance with shot 2, which
    # is not among them, so that instance stays fixed
    scene = _chain(instances=[0, 1, 2, 2, 3, 4])
    lp = ba_helpers.shot_poses_problem(scene, [1, 3])
    assert lp.interior == {1, 3} and lp.boundary == set()
    assert lp.free_instances == [1]
    # shot 1 sees points 10..34, shot 3 points 30..54
    np.testing.assert_array_equal(lp.point_ids, np.arange(10, 55))
    L, h = lp.adjuster._L, lp.adjuster._h
    assert int(L.gbba_num_projections(h)) == 50
