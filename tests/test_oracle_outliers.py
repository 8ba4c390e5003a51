"""The oracle's restatement of the outlier test of sfm::BAHelpers::RemoveOutliers
(ba_helpers.cc:1847-1975) on a hand-checked example."""
import numpy as np

from oracle import oracle


def test_auto_threshold_hand_example():
    # x: -1 0 0 1 3 -> median 0; y: -1 0 0 1 2 -> median 0; deviation norms
    # 0 1 2 sqrt(10) sqrt(2) -> median sqrt(2); robust std = 1.486 sqrt(2);
    # threshold = 3 |(std, std)| = 3 * 1.486 * 2 = 8.916
    e = np.array([[0.0, 0.0], [1.0, 0.0], [0.0, 2.0], [3.0, 1.0], [-1.0, -1.0]])
    w = np.array([1.0, 1.0, 1.0, 0.2, 1.0])
    pts = np.array([0, 0, 1, 1, 2])
    thr, flags, removed = oracle.remove_outliers(e, w, pts, 3, filter_type="AUTO")
    assert abs(thr - 8.916) < 1e-12
    np.testing.assert_array_equal(flags, [False, False, False, True, False])
    # point 1 keeps one observation; point 2 lost none
    np.testing.assert_array_equal(removed, [False, True, False])


def test_fixed_threshold_and_empty():
    e = np.array([[0.005, 0.0], [0.0, 0.007], [0.004, 0.004]])
    thr, flags, removed = oracle.remove_outliers(e, np.ones(3), np.array([0, 0, 0]), 1, filter_type="FIXED",
                                                 fixed_threshold=0.006)
    assert thr == 0.006
    np.testing.assert_array_equal(flags, [False, True, False])
    assert not removed[0]  # two observations remain
    thr, flags, removed = oracle.remove_outliers(np.zeros((0, 2)), np.zeros(0), np.zeros(0, int), 0,
                                                 filter_type="AUTO")
    assert thr == 1.0 and len(flags) == 0
