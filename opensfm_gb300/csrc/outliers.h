// Post-solve outlier selection: the observation test of
// sfm::BAHelpers::RemoveOutliers (ba_helpers.cc:1847-1975) on the device.
#pragma once

#include <cstdint>
#include <vector>

namespace gbba {

struct OutlierConfig {
  int filter_type = 0;             // 0 FIXED, 1 AUTO (bundle_outlier_filtering_type)
  double fixed_threshold = 0.006;  // bundle_outlier_fixed_threshold
  double auto_ratio = 3.0;         // bundle_outlier_auto_ratio
  double weight_threshold = 0.5;   // bundle_outlier_weight_threshold
};

struct OutlierResult {
  double threshold = 1.0;
  int64_t n_outliers = 0;
  int64_t n_removed_points = 0;
  double device_seconds = 0.0;  // CUDA-event span of the selection (inputs resident to flags written)
};

// errors: n rows of `stride` doubles (the first two are the 2D reprojection
// error), weights: n IRLS weights, obs_point: the point of every observation
// (n_points points).  Host arrays.  Writes flags[n] (1: outlier) and
// point_removed[n_points] (1: the point lost an observation and keeps fewer
// than two).
OutlierResult find_outliers(const double* errors, int stride, const double* weights, const int32_t* obs_point,
                            int64_t n, int64_t n_points, const OutlierConfig& cfg, uint8_t* flags,
                            uint8_t* point_removed);

}  // namespace gbba
