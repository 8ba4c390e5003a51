"""Device outlier selection against the oracle's numpy restatement of
sfm::BAHelpers::RemoveOutliers (ba_helpers.cc:1847-1975): thresholds and
flags are exact (radix-selected medians, uncontracted products)."""
import numpy as np
import pytest

from oracle import oracle
from opensfm_gb300 import outliers
from opensfm_gb300 import synthetic as syn
from opensfm_gb300.pybundle import adjuster_from_scene

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [1, 2, 7, 1000, 100001])
@pytest.mark.parametrize("filter_type", ["AUTO", "FIXED"])
def test_find_outliers_matches_oracle(n, filter_type):
    rng = np.random.default_rng(n)
    e = rng.standard_t(3, size=(n, 3)) * 1e-3
    e[rng.random(n) < 0.1] = 0.0  # ties, including at the median
    w = rng.random(n)
    n_points = max(1, n // 3)
    pts = rng.integers(0, n_points, n)
    thr, flags, removed = outliers.find_outliers(e, w, pts, n_points, filter_type=filter_type)
    thr_o, flags_o, removed_o = oracle.remove_outliers(e, w, pts, n_points, filter_type=filter_type)
    assert thr == thr_o
    np.testing.assert_array_equal(flags, flags_o)
    np.testing.assert_array_equal(removed, removed_o)


def test_negative_and_extreme_values():
    e = np.array([[-1e300, 2.0], [-0.0, 0.0], [5e-324, -7.0], [1e300, -1e-300], [-2.5, 3.5], [0.0, -0.0]])
    w = np.ones(6)
    pts = np.arange(6)
    thr, flags, removed = outliers.find_outliers(e, w, pts, 6, filter_type="AUTO")
    thr_o, flags_o, removed_o = oracle.remove_outliers(e, w, pts, 6, filter_type="AUTO")
    assert thr == thr_o
    np.testing.assert_array_equal(flags, flags_o)


def test_adjuster_outliers_after_irls():
    scene = syn.ring_scene(n_points=2000, outlier_ratio=0.03, seed=5)
    ba = adjuster_from_scene(scene, precision="mixed", irls="mixture", max_iterations=60, gps=False)
    ba.run()
    errs, w, _ = ba.projection_results()
    for ft in ("AUTO", "FIXED"):
        thr, flags, removed = ba.find_outliers(filter_type=ft)
        thr_o, flags_o, removed_o = oracle.remove_outliers(errs, w, scene.obs_point, len(scene.points),
                                                           filter_type=ft)
        assert thr == thr_o
        np.testing.assert_array_equal(flags, flags_o)
        np.testing.assert_array_equal(removed, removed_o)
    # the planted outliers (3%) are found: IRLS down-weights them
    assert 0.02 * len(w) < flags.sum() < 0.1 * len(w)
