"""Coarse space of the two-level PCG preconditioner, host side (no GPU):
spatial clusters of the rig instances and the distance-2 colouring of their
coupling graph, which makes the probed coarse matrix exact
(opensfm_gb300/csrc/coarse_space.cpp)."""
import numpy as np
import pytest

from opensfm_gb300 import synthetic as syn
from opensfm_gb300.pybundle import adjuster_from_scene


def cluster_graph(scene, cluster):
    obs_c = cluster[np.asarray(scene.obs_shot)]
    pts = np.asarray(scene.obs_point)
    n = cluster.max() + 1
    adj = np.zeros((n, n), bool)
    order = np.argsort(pts, kind="stable")
    starts = np.searchsorted(pts[order], np.arange(len(scene.points) + 1))
    for p in range(len(scene.points)):
        cs = np.unique(obs_c[order[starts[p]:starts[p + 1]]])
        adj[np.ix_(cs, cs)] = True
    np.fill_diagonal(adj, False)
    return adj


@pytest.mark.parametrize("leaf,nx,n_points", [(4, 12, 3000), (8, 12, 3000), (16, 12, 3000), (8, 24, 24000)])
def test_aerial_clusters_and_distance2_colouring(leaf, nx, n_points):
    # the larger case (about 200k observations) builds the coupling graph on
    # several host threads
    scene = syn.aerial_scene(seed=3, nx=nx, ny=nx, n_points=n_points)
    ba = adjuster_from_scene(scene, precision="fp64")
    n_inst = len(scene.rig_instance_poses)
    cluster, colour, n_col = ba.coarse_space_layout(leaf, n_inst)
    nc = len(colour)
    assert cluster.min() == 0 and cluster.max() == nc - 1
    sizes = np.bincount(cluster)
    assert sizes.max() <= leaf and sizes.min() >= leaf // 2 - 1
    assert nc >= n_inst // leaf
    # clusters are compact: the median cluster spans a few camera spacings
    c = scene.rig_instance_poses[:, 3:]
    span = np.median([np.ptp(c[cluster == k, :2], axis=0).max() for k in range(nc)])
    spacing = np.median(np.linalg.norm(np.diff(c[:nx, :2], axis=0), axis=1))
    assert span <= 2.0 * np.sqrt(leaf) * spacing
    # distance-2 colouring: within every closed neighbourhood each colour once
    adj = cluster_graph(scene, cluster)
    assert n_col == colour.max() + 1
    for k in range(nc):
        hood = np.concatenate([[k], np.nonzero(adj[k])[0]])
        assert len(np.unique(colour[hood])) == len(hood), k


def test_street_clusters_follow_the_trajectory():
    scene = syn.street_scene(n_shots=120, n_points=4000, seed=5, outlier_ratio=0.0)
    ba = adjuster_from_scene(scene, precision="fp64")
    cluster, colour, n_col = ba.coarse_space_layout(10, 120)
    # shots are numbered along the street: a cluster is a run of neighbours
    for k in range(len(colour)):
        idx = np.nonzero(cluster == k)[0]
        assert idx.max() - idx.min() < 3 * len(idx)
    adj = cluster_graph(scene, cluster)
    for k in range(len(colour)):
        hood = np.concatenate([[k], np.nonzero(adj[k])[0]])
        assert len(np.unique(colour[hood])) == len(hood)


def test_small_problems_get_no_coarse_space_and_bad_sizes_are_refused():
    scene = syn.aerial_scene(seed=3, nx=6, ny=6, n_points=800)
    ba = adjuster_from_scene(scene, precision="fp64")
    # a problem too small for two clusters gets none
    cluster, colour, _ = ba.coarse_space_layout(1000, 36)
    assert len(colour) == 0 and np.all(cluster == -1)
    with pytest.raises(Exception):
        ba.coarse_space_layout(0, 36)
    with pytest.raises(Exception):
        ba.set_coarse_preconditioner(-1)
    with pytest.raises(Exception):
        ba.coarse_space_layout(4, 35)


def test_fixed_instances_join_no_cluster():
    scene = syn.aerial_scene(seed=3, nx=8, ny=8, n_points=1500)
    fixed = [0, 9, 27, 63]
    ba = adjuster_from_scene(scene, precision="fp64", fixed_instances=fixed)
    cluster, colour, _ = ba.coarse_space_layout(6, 64)
    assert np.all(cluster[fixed] == -1)
    free = np.setdiff1d(np.arange(64), fixed)
    assert np.all(cluster[free] >= 0)
    assert np.bincount(cluster[free]).max() <= 6


def test_host_terms_couple_their_clusters():
    # a common-position term between shots of two clusters that share a
    # colour ties those clusters: afterwards their colours differ, and every
    # closed neighbourhood (observations and host terms) stays distinct
    scene = syn.aerial_scene(seed=3, nx=12, ny=12, n_points=3000)
    ba = adjuster_from_scene(scene, precision="fp64")
    cluster0, colour0, _ = ba.coarse_space_layout(8, 144)
    a = 0
    b = int(np.nonzero((colour0 == colour0[a]) & (np.arange(len(colour0)) != a))[0][-1])
    sa, sb = int(np.nonzero(cluster0 == a)[0][0]), int(np.nonzero(cluster0 == b)[0][0])
    ba.add_common_position(str(sa), str(sb), 1.0, 0.1)
    cluster, colour, _ = ba.coarse_space_layout(8, 144)
    np.testing.assert_array_equal(cluster, cluster0)  # the clusters depend on the centres only
    assert colour[a] != colour[b]
    adj = cluster_graph(scene, cluster)
    adj[a, b] = adj[b, a] = True
    for k in range(len(colour)):
        hood = np.concatenate([[k], np.nonzero(adj[k])[0]])
        assert len(np.unique(colour[hood])) == len(hood)
