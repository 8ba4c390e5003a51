// extern "C" entry points of the bundle adjuster (include/gbba.h).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <memory>
#include <string>
#include <vector>

#include "../../include/gbba.h"
#include "adjuster.h"
#include "capi_util.h"
#include "solver.h"

struct gbba_adjuster {
  gbba::BundleAdjuster ba;
};

using gbba::ApiError;
using gbba::guarded;

namespace {

gbba::BundleAdjuster& ba_of(gbba_adjuster_t* h) {
  if (!h) throw ApiError(GBBA_ERR_INVALID_ARGUMENT, "adjuster handle is NULL");
  return h->ba;
}
const gbba::BundleAdjuster& ba_of(const gbba_adjuster_t* h) {
  if (!h) throw ApiError(GBBA_ERR_INVALID_ARGUMENT, "adjuster handle is NULL");
  return h->ba;
}
std::string str(const char* s) {
  if (!s) throw ApiError(GBBA_ERR_INVALID_ARGUMENT, "string argument is NULL");
  return std::string(s);
}
template <typename T>
void need(const T* p, const char* what) {
  if (!p) throw ApiError(GBBA_ERR_INVALID_ARGUMENT, std::string(what) + " is NULL");
}
int copy_string(const std::string& s, char* buf, size_t len) {
  if (buf && len) {
    const size_t n = std::min(len - 1, s.size());
    std::memcpy(buf, s.data(), n);
    buf[n] = '\0';
  }
  return int(s.size());
}

}  // namespace

extern "C" {

gbba_adjuster_t* gbba_create(void) {
  gbba_adjuster_t* h = nullptr;
  guarded([&] { h = new gbba_adjuster_t; });
  return h;
}

void gbba_destroy(gbba_adjuster_t* h) { delete h; }

int gbba_add_camera(gbba_adjuster_t* h, const char* id, int projection, const double* values,
                    const double* prior_values, int n_values, int constant) {
  return guarded([&] {
    need(values, "values");
    need(prior_values, "prior_values");
    try {
      ba_of(h).AddCamera(str(id), projection, values, prior_values, n_values, constant != 0);
    } catch (const std::invalid_argument& e) {
      throw ApiError(GBBA_ERR_INVALID_ARGUMENT, e.what());
    }
  });
}

int gbba_set_camera_bias(gbba_adjuster_t* h, const char* camera_id, const double* rotation,
                         const double* translation, double scale) {
  return guarded([&] {
    need(rotation, "rotation");
    need(translation, "translation");
    ba_of(h).SetCameraBias(str(camera_id), rotation, translation, scale);
  });
}

int gbba_set_camera_bias_parameters(gbba_adjuster_t* h, const char* camera_id, const int* indices, int n) {
  return guarded([&] {
    if (n < 0) throw ApiError(GBBA_ERR_INVALID_ARGUMENT, "negative bias parameter count");
    if (n > 0) need(indices, "indices");
    ba_of(h).SetCameraBiasParameters(str(camera_id), indices, n);
  });
}

int gbba_get_bias(const gbba_adjuster_t* h, const char* camera_id, double* rotation, double* translation,
                  double* scale) {
  return guarded([&] {
    need(rotation, "rotation");
    need(translation, "translation");
    need(scale, "scale");
    ba_of(h).GetBias(str(camera_id), rotation, translation, scale);
  });
}

int gbba_add_rig_camera(gbba_adjuster_t* h, const char* id, const double* pose, const double* pose_prior, int fixed) {
  return guarded([&] {
    need(pose, "pose");
    need(pose_prior, "pose_prior");
    ba_of(h).AddRigCamera(str(id), pose, pose_prior, fixed != 0);
  });
}

int gbba_add_rig_instance(gbba_adjuster_t* h, const char* id, const double* pose, int n_shots,
                          const char* const* shot_ids, const char* const* camera_ids,
                          const char* const* rig_camera_ids, int fixed) {
  return guarded([&] {
    need(pose, "pose");
    if (n_shots < 0) throw ApiError(GBBA_ERR_INVALID_ARGUMENT, "negative shot count");
    std::vector<std::string> s, c, r;
    for (int i = 0; i < n_shots; ++i) {
      s.push_back(str(shot_ids[i]));
      c.push_back(str(camera_ids[i]));
      r.push_back(str(rig_camera_ids[i]));
    }
    ba_of(h).AddRigInstance(str(id), pose, s, c, r, fixed != 0);
  });
}

int gbba_add_rig_instance_position_prior(gbba_adjuster_t* h, const char* id, const double* position,
                                         const double* std_dev, const char* scale_group) {
  return guarded([&] {
    need(position, "position");
    need(std_dev, "std_dev");
    ba_of(h).AddRigInstancePositionPrior(str(id), position, std_dev, scale_group ? scale_group : "");
  });
}

int gbba_add_point(gbba_adjuster_t* h, const char* id, const double* position, int constant) {
  return guarded([&] {
    need(position, "position");
    ba_of(h).AddPoint(str(id), position, constant != 0);
  });
}

int gbba_add_absolute_up_vector(gbba_adjuster_t* h, const char* shot_id, const double* up_vector,
                                double std_deviation) {
  return guarded([&] {
    need(up_vector, "up_vector");
    ba_of(h).AddOrientationConstraint(str(shot_id), gbba::OrientationTerm::kUpVector, up_vector, std_deviation);
  });
}

int gbba_orientation_residual(int kind, const double* target, double std_deviation,
                              const double* instance_rotation, const double* camera_rotation, double* residuals,
                              double* jacobian, int* n_residuals) {
  return guarded([&] {
    if (kind < 0 || kind > 3 || !target || !instance_rotation || !residuals || !jacobian || !n_residuals ||
        !(std_deviation > 0.0))
      throw gbba::ApiError(GBBA_ERR_INVALID_ARGUMENT, "gbba_orientation_residual: invalid argument");
    gbba::OrientationTerm t;
    t.kind = kind;
    t.rig_camera = camera_rotation ? 0 : -1;
    t.scale = 1.0 / std_deviation;
    if (kind == gbba::OrientationTerm::kUpVector) {
      const double n = std::sqrt(target[0] * target[0] + target[1] * target[1] + target[2] * target[2]);
      if (!(n > 0.0)) throw gbba::ApiError(GBBA_ERR_INVALID_ARGUMENT, "gbba_orientation_residual: zero up vector");
      for (int k = 0; k < 3; ++k) t.target[k] = target[k] / n;
    } else {
      t.target[0] = target[0];
    }
    gbba::orient::D r[3];
    const int m = gbba::orient::residuals(t, instance_rotation, camera_rotation, r);
    for (int q = 0; q < m; ++q) {
      residuals[q] = r[q].v;
      for (int k = 0; k < 6; ++k) jacobian[6 * q + k] = r[q].d[k];
    }
    *n_residuals = m;
  });
}

int gbba_add_relative_rotation(gbba_adjuster_t* h, const char* shot_i, const char* shot_j, const double* rotation,
                               const double* scale_matrix) {
  return guarded([&] {
    need(rotation, "rotation");
    ba_of(h).AddRelativeRotation(str(shot_i), str(shot_j), rotation, scale_matrix);
  });
}

int gbba_add_common_position(gbba_adjuster_t* h, const char* shot_i, const char* shot_j, double margin,
                             double std_deviation) {
  return guarded([&] { ba_of(h).AddCommonPosition(str(shot_i), str(shot_j), margin, std_deviation); });
}

int gbba_add_linear_motion(gbba_adjuster_t* h, const char* shot0, const char* shot1, const char* shot2,
                           double alpha, double position_std_deviation, double orientation_std_deviation) {
  return guarded([&] {
    ba_of(h).AddLinearMotion(str(shot0), str(shot1), str(shot2), alpha, position_std_deviation,
                             orientation_std_deviation);
  });
}

int gbba_set_relative_motion_loss_function(gbba_adjuster_t* h, const char* name, double threshold) {
  return guarded([&] { ba_of(h).SetRelativeMotionLossFunction(str(name), threshold); });
}

int gbba_set_gauge_fix_shots(gbba_adjuster_t* h, const char* shot_origin, const char* shot_scale) {
  return guarded([&] { ba_of(h).SetGaugeFixShots(str(shot_origin), str(shot_scale)); });
}

int gbba_add_heatmap(gbba_adjuster_t* h, const char* heatmap_id, const double* data, int64_t n, int64_t width,
                     double resolution) {
  return guarded([&] {
    need(data, "data");
    try {
      ba_of(h).AddHeatmap(str(heatmap_id), data, n, width, resolution);
    } catch (const std::invalid_argument& e) {
      throw gbba::ApiError(GBBA_ERR_INVALID_ARGUMENT, e.what());
    }
  });
}

int gbba_add_absolute_position_heatmap(gbba_adjuster_t* h, const char* shot_id, const char* heatmap_id,
                                       double x_offset, double y_offset, double std_deviation) {
  return guarded([&] {
    ba_of(h).AddAbsolutePositionHeatmap(str(shot_id), str(heatmap_id), x_offset, y_offset, std_deviation);
  });
}

int gbba_host_loss(int kind, double a, double s, double* rho) {
  return guarded([&] {
    if (kind < 0 || kind > 5 || !rho || !(a > 0.0))
      throw gbba::ApiError(GBBA_ERR_INVALID_ARGUMENT, "gbba_host_loss: invalid argument");
    gbba::orient::loss_rho(kind, a, s, rho);
  });
}

int gbba_heatmap_residual(const double* grid, int64_t n, int64_t width, double resolution, double x_offset,
                          double y_offset, double std_deviation, const double* instance_pose,
                          const double* rig_camera_pose, double* residual, double* jacobian) {
  return guarded([&] {
    if (!grid || width <= 0 || n < width || n % width != 0 || !instance_pose || !residual || !jacobian)
      throw gbba::ApiError(GBBA_ERR_INVALID_ARGUMENT, "gbba_heatmap_residual: invalid argument");
    gbba::RelativeTerm t;
    t.kind = gbba::RelativeTerm::kHeatmap;
    t.n_shots = 1;
    t.grid.data = grid;
    t.grid.width = int(width);
    t.grid.height = int(n / width);
    t.grid.resolution = resolution;
    t.x_offset = x_offset;
    t.y_offset = y_offset;
    t.scale = 1.0 / std_deviation;
    const double* pi[3] = {instance_pose, nullptr, nullptr};
    const double* pc[3] = {rig_camera_pose, nullptr, nullptr};
    gbba::orient::Dual<12> r[7];
    gbba::orient::relative_residuals<12>(t, pi, pc, r);
    residual[0] = r[0].v;
    for (int k = 0; k < 12; ++k) jacobian[k] = r[0].d[k];
  });
}

int gbba_add_reconstruction(gbba_adjuster_t* h, const char* id, int constant) {
  return guarded([&] { ba_of(h).AddReconstruction(str(id), constant != 0); });
}

int gbba_add_reconstruction_instance(gbba_adjuster_t* h, const char* reconstruction_id, double scale,
                                     const char* instance_id) {
  return guarded([&] { ba_of(h).AddReconstructionInstance(str(reconstruction_id), scale, str(instance_id)); });
}

int gbba_set_scale_sharing(gbba_adjuster_t* h, const char* id, int share) {
  return guarded([&] { ba_of(h).SetScaleSharing(str(id), share != 0); });
}

int gbba_get_reconstruction_scale(const gbba_adjuster_t* h, const char* reconstruction_id, const char* instance_id,
                                  double* scale) {
  return guarded([&] {
    need(scale, "scale");
    *scale = ba_of(h).GetReconstructionScale(str(reconstruction_id), str(instance_id));
  });
}

int gbba_set_adjust_absolute_position_std(gbba_adjuster_t* h, int adjust) {
  return guarded([&] { ba_of(h).SetAdjustAbsolutePositionStd(adjust != 0); });
}

int gbba_has_reconstruction(const gbba_adjuster_t* h, const char* reconstruction_id) {
  int has = 0;
  const int st = guarded([&] { has = ba_of(h).HasReconstruction(str(reconstruction_id)) ? 1 : 0; });
  return st == GBBA_OK ? has : -1;
}

int gbba_add_relative_motion(gbba_adjuster_t* h, const char* instance_i, const char* instance_j,
                             const double* motion, double robust_multiplier, int observed_scale,
                             const double* scale_matrix) {
  return guarded([&] {
    need(motion, "motion");
    ba_of(h).AddRelativeMotion(str(instance_i), str(instance_j), motion, robust_multiplier, observed_scale != 0,
                               scale_matrix);
  });
}

int gbba_relative_residual(int kind, const double* instance_poses, const double* rig_camera_poses,
                           const double* params, double* residuals, double* jacobian, int* n_residuals) {
  return guarded([&] {
    if (kind < 0 || kind > 8 || kind == 4 || !params || !residuals || !jacobian || !n_residuals ||
        (kind != 7 && !instance_poses))
      throw gbba::ApiError(GBBA_ERR_INVALID_ARGUMENT, "gbba_relative_residual: invalid argument");
    // kind 8: the GPS prior of kind 6 through an optimised camera bias
    const bool biased = kind == 8;
    if (biased) kind = gbba::RelativeTerm::kGpsStd;
    double bias[7] = {0, 0, 0, 0, 0, 0, 1};
    gbba::RelativeTerm t;
    t.kind = kind;
    t.n_shots = kind == gbba::RelativeTerm::kLinearMotion ? 3
                : kind == gbba::RelativeTerm::kGpsStd          ? 1
                : kind == gbba::RelativeTerm::kStdDeviation    ? 0
                                                               : 2;
    double scales[2] = {1.0, 1.0};
    if (kind == gbba::RelativeTerm::kRelativeRotation) {
      for (int k = 0; k < 3; ++k) t.rotation[k] = params[k];
      for (int k = 0; k < 9; ++k) t.scale_matrix[k] = params[3 + k];
    } else if (kind == gbba::RelativeTerm::kCommonPosition) {
      t.margin = params[0];
      t.scale = 1.0 / params[1];
    } else if (kind == gbba::RelativeTerm::kGaugeScale) {
      t.distance = params[0];
    } else if (kind == gbba::RelativeTerm::kRelativeMotion) {
      for (int k = 0; k < 7; ++k) t.motion[k] = params[k];
      t.observed_scale = params[7] != 0.0;
      for (int k = 0; k < 49; ++k) t.motion_matrix[k] = params[8 + k];
      scales[0] = params[57];
      scales[1] = params[58];
    } else if (kind == gbba::RelativeTerm::kGpsStd) {
      for (int k = 0; k < 3; ++k) {
        t.prior[k] = params[k];
        // DataPriorError's 1 / max(sigma, epsilon) (prior_error.h:27-36)
        t.prior_scale[k] = 1.0 / std::max(params[3 + k], std::numeric_limits<double>::epsilon());
      }
      scales[0] = params[6];
      if (biased)
        for (int k = 0; k < 7; ++k) bias[k] = params[7 + k];
    } else if (kind == gbba::RelativeTerm::kStdDeviation) {
      scales[0] = params[0];
    } else {
      t.alpha = params[0];
      t.position_scale = 1.0 / params[1];
      t.orientation_scale = 1.0 / params[2];
    }
    const double* pi[3] = {nullptr, nullptr, nullptr};
    const double* pc[3] = {nullptr, nullptr, nullptr};
    for (int k = 0; k < t.n_shots; ++k) {
      pi[k] = instance_poses + 6 * k;
      pc[k] = rig_camera_poses ? rig_camera_poses + 6 * k : nullptr;
    }
    gbba::orient::Dual<36> r[7];
    const int m = gbba::orient::relative_residuals<36>(t, pi, pc, r, scales, biased ? bias : nullptr);
    for (int q = 0; q < m; ++q) {
      residuals[q] = r[q].v;
      for (int k = 0; k < 36; ++k) jacobian[36 * q + k] = r[q].d[k];
    }
    *n_residuals = m;
  });
}

static int add_angle(gbba_adjuster_t* h, const char* shot_id, int kind, double angle, double std_deviation) {
  return guarded([&] { ba_of(h).AddOrientationConstraint(str(shot_id), kind, &angle, std_deviation); });
}
int gbba_add_absolute_pan(gbba_adjuster_t* h, const char* shot_id, double angle, double std_deviation) {
  return add_angle(h, shot_id, gbba::OrientationTerm::kPan, angle, std_deviation);
}
int gbba_add_absolute_tilt(gbba_adjuster_t* h, const char* shot_id, double angle, double std_deviation) {
  return add_angle(h, shot_id, gbba::OrientationTerm::kTilt, angle, std_deviation);
}
int gbba_add_absolute_roll(gbba_adjuster_t* h, const char* shot_id, double angle, double std_deviation) {
  return add_angle(h, shot_id, gbba::OrientationTerm::kRoll, angle, std_deviation);
}

int gbba_add_point_prior(gbba_adjuster_t* h, const char* id, const double* position, const double* std_dev,
                         int has_altitude) {
  return guarded([&] {
    need(position, "position");
    need(std_dev, "std_dev");
    ba_of(h).AddPointPrior(str(id), position, std_dev, has_altitude != 0);
  });
}

int gbba_add_point_projection_observation(gbba_adjuster_t* h, const char* shot, const char* point,
                                          const double* observation, double std_dev, int is_gcp) {
  return guarded([&] {
    need(observation, "observation");
    ba_of(h).AddPointProjectionObservation(str(shot), str(point), observation, std_dev, is_gcp != 0);
  });
}

int gbba_set_observation_depth_priors(gbba_adjuster_t* h, int64_t n, const int64_t* observation_index,
                                      const double* value, const double* std_dev, const uint8_t* is_radial) {
  return guarded([&] {
    if (n < 0) throw ApiError(GBBA_ERR_INVALID_ARGUMENT, "negative depth prior count");
    if (n == 0) return;
    need(observation_index, "observation_index");
    need(value, "value");
    need(std_dev, "std_dev");
    auto& ba = ba_of(h);
    // check every entry before attaching any
    for (int64_t i = 0; i < n; ++i) {
      if (observation_index[i] < 0 || observation_index[i] >= ba.NumObservations())
        throw std::out_of_range("depth prior " + std::to_string(i) + " references an unknown observation");
      if (!(std_dev[i] > 0.0))
        throw ApiError(GBBA_ERR_INVALID_ARGUMENT, "depth prior " + std::to_string(i) + ": std deviation must be positive");
    }
    for (int64_t i = 0; i < n; ++i)
      ba.SetObservationDepthPrior(observation_index[i], value[i], std_dev[i], is_radial ? is_radial[i] != 0 : true);
  });
}

int64_t gbba_shot_index(const gbba_adjuster_t* h, const char* shot) {
  int64_t r = -1;
  guarded([&] { r = ba_of(h).ShotIndex(str(shot)); });
  return r;
}

int64_t gbba_point_index(const gbba_adjuster_t* h, const char* point) {
  int64_t r = -1;
  guarded([&] { r = ba_of(h).PointIndex(str(point)); });
  return r;
}

int gbba_add_points_bulk(gbba_adjuster_t* h, int64_t n, const double* xyz, const uint8_t* constant,
                         const char* const* ids, int64_t* first_index) {
  return guarded([&] {
    if (n < 0) throw ApiError(GBBA_ERR_INVALID_ARGUMENT, "negative point count");
    if (n) need(xyz, "xyz");
    const int64_t f = ba_of(h).AddPointsBulk(n, xyz, constant, ids);
    if (first_index) *first_index = f;
  });
}

int gbba_add_point_projection_observations_bulk(gbba_adjuster_t* h, int64_t n, const int32_t* shot_index,
                                                const int32_t* point_index, const double* xy,
                                                const double* std_dev, const uint8_t* is_gcp) {
  return guarded([&] {
    if (n < 0) throw ApiError(GBBA_ERR_INVALID_ARGUMENT, "negative observation count");
    if (n) {
      need(shot_index, "shot_index");
      need(point_index, "point_index");
      need(xy, "xy");
      need(std_dev, "std_dev");
    }
    try {
      ba_of(h).AddObservationsBulk(n, shot_index, point_index, xy, std_dev, is_gcp);
    } catch (const std::invalid_argument& e) {
      throw ApiError(GBBA_ERR_INVALID_ARGUMENT, e.what());
    }
  });
}

int gbba_set_point_projection_loss_function(gbba_adjuster_t* h, const char* name, double threshold) {
  return guarded([&] { ba_of(h).SetPointProjectionLossFunction(str(name), threshold); });
}

int gbba_set_irls_mode(gbba_adjuster_t* h, int mode) {
  return guarded([&] {
    if (mode != 0 && mode != 1) throw ApiError(GBBA_ERR_INVALID_ARGUMENT, "IRLS mode must be 0 (none) or 1 (mixture)");
    ba_of(h).SetIrlsMode(mode);
  });
}

int gbba_set_precision(gbba_adjuster_t* h, int precision) {
  return guarded([&] {
    if (precision != GBBA_PRECISION_FP64 && precision != GBBA_PRECISION_MIXED)
      throw ApiError(GBBA_ERR_INVALID_ARGUMENT, "unknown precision");
    ba_of(h).SetPrecision(precision);
  });
}

int gbba_set_max_num_iterations(gbba_adjuster_t* h, int n) {
  return guarded([&] { ba_of(h).SetMaxNumIterations(n); });
}

int gbba_set_num_threads(gbba_adjuster_t* h, int n) {
  return guarded([&] { ba_of(h).SetNumThreads(n); });
}

int gbba_set_use_analytic_derivatives(gbba_adjuster_t* h, int use) {
  return guarded([&] { ba_of(h).SetUseAnalyticDerivatives(use != 0); });
}

int gbba_set_linear_solver_type(gbba_adjuster_t* h, const char* type) {
  return guarded([&] { ba_of(h).SetLinearSolverType(str(type)); });
}

int gbba_set_internal_parameters_prior_sd(gbba_adjuster_t* h, double focal_sd, double aspect_ratio_sd, double c_sd,
                                          double k1_sd, double k2_sd, double p1_sd, double p2_sd, double k3_sd,
                                          double k4_sd) {
  return guarded([&] {
    ba_of(h).SetInternalParametersPriorSD(focal_sd, aspect_ratio_sd, c_sd, k1_sd, k2_sd, p1_sd, p2_sd, k3_sd, k4_sd);
  });
}

int gbba_set_rig_parameters_prior_sd(gbba_adjuster_t* h, double translation_sd, double rotation_sd) {
  return guarded([&] { ba_of(h).SetRigParametersPriorSD(translation_sd, rotation_sd); });
}

int gbba_set_compute_reprojection_errors(gbba_adjuster_t* h, int v) {
  return guarded([&] { ba_of(h).SetComputeReprojectionErrors(v != 0); });
}

int gbba_set_compute_covariances(gbba_adjuster_t* h, int v) {
  return guarded([&] { ba_of(h).SetComputeCovariances(v != 0); });
}

int gbba_get_rig_instance_covariance(const gbba_adjuster_t* h, const char* id, double* out) {
  return guarded([&] {
    need(out, "out");
    ba_of(h).GetRigInstanceCovariance(str(id), out);
  });
}

int gbba_get_covariance_estimation_valid(const gbba_adjuster_t* h) {
  int v = 0;
  guarded([&] { v = ba_of(h).CovarianceValid() ? 1 : 0; });
  return v;
}

int gbba_set_skip_initial_reweighting(gbba_adjuster_t* h, int v) {
  return guarded([&] { ba_of(h).SetSkipInitialReweighting(v != 0); });
}

int gbba_set_default_density_ratio(gbba_adjuster_t* h, double ratio) {
  return guarded([&] { ba_of(h).SetDefaultDensityRatio(ratio); });
}

double gbba_get_default_density_ratio(const gbba_adjuster_t* h) {
  double v = 0.0;
  guarded([&] { v = ba_of(h).GetDefaultDensityRatio(); });
  return v;
}

int gbba_set_group_density_ratio(gbba_adjuster_t* h, const char* group, double ratio) {
  return guarded([&] { ba_of(h).SetGroupDensityRatio(str(group), ratio); });
}

double gbba_get_group_density_ratio(const gbba_adjuster_t* h, const char* group) {
  double v = 0.0;
  guarded([&] { v = ba_of(h).GetGroupDensityRatio(str(group)); });
  return v;
}

int gbba_set_pcg_graph(gbba_adjuster_t* h, int enable) {
  return guarded([&] { ba_of(h).SetPcgGraph(enable != 0); });
}

int gbba_set_coarse_preconditioner(gbba_adjuster_t* h, int leaf) {
  return guarded([&] {
    if (leaf < 0) throw ApiError(GBBA_ERR_INVALID_ARGUMENT, "coarse cluster size must be >= 0");
    ba_of(h).SetCoarsePreconditioner(leaf);
  });
}

int gbba_get_coarse_info(const gbba_adjuster_t* h, int* clusters, int* colours, int64_t* probes) {
  return guarded([&] {
    const gbba::SolveSummary& s = ba_of(h).Summary();
    if (clusters) *clusters = s.coarse_clusters;
    if (colours) *colours = s.coarse_colours;
    if (probes) *probes = s.coarse_probes;
  });
}

int gbba_coarse_space_layout(gbba_adjuster_t* h, int leaf, int* cluster_of_instance, int64_t n_instances,
                             int* colour_of_cluster, int cluster_capacity, int* clusters, int* colours) {
  return guarded([&] {
    if (leaf < 1) throw ApiError(GBBA_ERR_INVALID_ARGUMENT, "coarse cluster size must be >= 1");
    const gbba::CoarseSpace cs = ba_of(h).CoarseLayout(leaf);
    if (n_instances != int64_t(cs.cluster.size()))
      throw ApiError(GBBA_ERR_INVALID_ARGUMENT, "cluster_of_instance must hold one entry per rig instance");
    need(cluster_of_instance, "cluster_of_instance");
    std::copy(cs.cluster.begin(), cs.cluster.end(), cluster_of_instance);
    if (colour_of_cluster)
      for (int c = 0; c < std::min(cluster_capacity, cs.n_clusters); ++c) colour_of_cluster[c] = cs.colour[c];
    if (clusters) *clusters = cs.n_clusters;
    if (colours) *colours = cs.n_colours;
  });
}

int gbba_set_matrix_free(gbba_adjuster_t* h, int mode) {
  return guarded([&] {
    if (mode < -1 || mode > 1) throw ApiError(GBBA_ERR_INVALID_ARGUMENT, "matrix-free mode must be -1, 0 or 1");
    ba_of(h).SetMatrixFree(mode);
  });
}

int gbba_set_pcg_tolerance(gbba_adjuster_t* h, double tolerance) {
  return guarded([&] {
    if (!(tolerance > 0.0)) throw ApiError(GBBA_ERR_INVALID_ARGUMENT, "tolerance must be positive");
    ba_of(h).SetPcgTolerance(tolerance);
  });
}

int gbba_set_shard(gbba_adjuster_t* h, int rank, int world_size, gbba_allreduce_fn allreduce, void* ctx) {
  return guarded([&] {
    try {
      ba_of(h).SetShard(rank, world_size, allreduce, ctx);
    } catch (const std::invalid_argument& e) {
      throw ApiError(GBBA_ERR_INVALID_ARGUMENT, e.what());
    }
  });
}

int gbba_get_shard_points(const gbba_adjuster_t* h, int rank, int64_t* first, int64_t* last) {
  return guarded([&] {
    need(first, "first");
    need(last, "last");
    const gbba::BundleAdjuster& ba = ba_of(h);
    if (rank < 0 || rank >= ba.Shard().world) throw ApiError(GBBA_ERR_INVALID_ARGUMENT, "rank out of range");
    const auto r = ba.ShardRange(rank);
    *first = r.first;
    *last = r.second;
  });
}

int gbba_run(gbba_adjuster_t* h) {
  return guarded([&] { ba_of(h).Run(); });
}

int gbba_get_camera(const gbba_adjuster_t* h, const char* id, int* projection, double* values, int capacity,
                    int* n_values) {
  return guarded([&] {
    need(values, "values");
    const int n = ba_of(h).GetCamera(str(id), projection, values, capacity);
    if (n_values) *n_values = n;
  });
}

int gbba_get_rig_instance_pose(const gbba_adjuster_t* h, const char* id, double* pose) {
  return guarded([&] {
    need(pose, "pose");
    ba_of(h).GetRigInstancePose(str(id), pose);
  });
}

int gbba_get_rig_camera_pose(const gbba_adjuster_t* h, const char* id, double* pose) {
  return guarded([&] {
    need(pose, "pose");
    ba_of(h).GetRigCameraPose(str(id), pose);
  });
}

int gbba_get_point(const gbba_adjuster_t* h, const char* id, double* position) {
  return guarded([&] {
    need(position, "position");
    ba_of(h).GetPoint(str(id), position);
  });
}

int gbba_has_point(const gbba_adjuster_t* h, const char* id) {
  int v = 0;
  guarded([&] { v = ba_of(h).HasPoint(str(id)) ? 1 : 0; });
  return v;
}

int64_t gbba_num_projections(const gbba_adjuster_t* h) {
  int64_t v = 0;
  guarded([&] { v = ba_of(h).NumProjections(); });
  return v;
}

int64_t gbba_num_points(const gbba_adjuster_t* h) {
  int64_t v = 0;
  guarded([&] { v = ba_of(h).NumPoints(); });
  return v;
}

int gbba_get_points_bulk(const gbba_adjuster_t* h, int64_t first, int64_t n, double* xyz) {
  return guarded([&] {
    if (n) need(xyz, "xyz");
    ba_of(h).GetPointsBulk(first, n, xyz);
  });
}

int gbba_get_projection_results(const gbba_adjuster_t* h, int64_t n, double* errors, double* weights, int32_t* dims) {
  return guarded([&] {
    if (n) need(errors, "errors");
    try {
      ba_of(h).GetProjectionResults(n, errors, weights, dims);
    } catch (const std::invalid_argument& e) {
      throw ApiError(GBBA_ERR_INVALID_ARGUMENT, e.what());
    }
  });
}

int gbba_adjuster_find_outliers(const gbba_adjuster_t* h, const gbba_outlier_config_t* config, uint8_t* flags,
                                uint8_t* point_removed, gbba_outlier_result_t* result) {
  const gbba::BundleAdjuster* ba = nullptr;
  int st = guarded([&] {
    ba = &ba_of(h);
    if (!ba->HasResults())
      throw ApiError(GBBA_ERR_RUNTIME, "no reprojection errors: run the adjuster (with reprojection errors) first");
  });
  if (st != GBBA_OK) return st;
  const std::vector<int32_t> pts = ba->ObservationPoints();
  return gbba_find_outliers(ba->Errors().data(), 3, ba->Weights().data(), pts.data(), ba->NumObservations(),
                            ba->NumPoints(), config, flags, point_removed, result);
}

int gbba_brief_report(const gbba_adjuster_t* h, char* buf, size_t len) {
  int n = 0;
  const int st = guarded([&] { n = copy_string(ba_of(h).BriefReport(), buf, len); });
  return st == GBBA_OK ? n : -1;
}

int gbba_full_report(const gbba_adjuster_t* h, char* buf, size_t len) {
  int n = 0;
  const int st = guarded([&] { n = copy_string(ba_of(h).FullReport(), buf, len); });
  return st == GBBA_OK ? n : -1;
}

int gbba_irls_report(const gbba_adjuster_t* h, char* buf, size_t len) {
  int n = 0;
  const int st = guarded([&] { n = copy_string(ba_of(h).IrlsReport(), buf, len); });
  return st == GBBA_OK ? n : -1;
}

int gbba_get_summary(const gbba_adjuster_t* h, gbba_summary_t* out) {
  return guarded([&] {
    need(out, "out");
    const gbba::SolveSummary& s = ba_of(h).Summary();
    out->initial_cost = s.initial_cost;
    out->final_cost = s.final_cost;
    out->seconds = s.seconds;
    out->linear_solver_seconds = s.linear_solver_seconds;
    out->jacobian_seconds = s.jacobian_seconds;
    out->residual_seconds = s.residual_seconds;
    out->iterations = s.iterations;
    out->successful_steps = s.successful_steps;
    out->unsuccessful_steps = s.unsuccessful_steps;
    out->kernel_launches = s.kernel_launches;
    out->setup_seconds = s.setup_seconds;
    out->linear_solver_failures = s.linear_solver_failures;
    out->usable = s.usable ? 1 : 0;
  });
}

int gbba_get_trace(const gbba_adjuster_t* h, int capacity, double* records, int* n) {
  return guarded([&] {
    const gbba::SolveSummary& s = ba_of(h).Summary();
    const int m = int(s.trace.size());
    if (n) *n = m;
    if (!records) return;
    for (int i = 0; i < std::min(capacity, m); ++i) {
      const gbba::IterationRecord& r = s.trace[i];
      double* o = records + 8 * int64_t(i);
      o[0] = r.iteration;
      o[1] = r.cost;
      o[2] = r.seconds;
      o[3] = r.success ? 1.0 : 0.0;
      o[4] = r.linear_iterations;
      o[5] = r.radius;
      o[6] = r.relative_decrease;
      o[7] = r.step_norm;
    }
  });
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Batched runs: many adjusters solved together on the device.

// relative residual of the batch's exact steps
constexpr double kBatchExactTolerance = 1e-10;

struct gbba_batch {
  std::vector<gbba_adjuster_t*> items;
  gbba::BatchOptions opts;
  int precision = 1;
  bool exact = false;  // exact steps (gbba_batch_set_linear_solver)
  gbba::BatchSummary summary;
  bool has_run = false;
};

extern "C" {

gbba_batch_t* gbba_batch_create(void) {
  gbba_batch_t* b = nullptr;
  guarded([&] { b = new gbba_batch_t(); });
  return b;
}

void gbba_batch_destroy(gbba_batch_t* b) { delete b; }

int gbba_batch_add(gbba_batch_t* b, gbba_adjuster_t* h) {
  return guarded([&] {
    if (!b) throw ApiError(GBBA_ERR_INVALID_ARGUMENT, "batch handle is NULL");
    if (ba_of(h).Shard().world > 1)
      throw ApiError(GBBA_ERR_INVALID_ARGUMENT, "a sharded adjuster cannot join a batch (the batch is single-rank)");
    b->items.push_back(h);
  });
}

int gbba_batch_size(const gbba_batch_t* b) { return b ? int(b->items.size()) : 0; }

int gbba_batch_set_options(gbba_batch_t* b, int precision, int max_iterations, int pcg_iterations,
                           double pcg_tolerance, int use_graph, int autotune) {
  return guarded([&] {
    if (!b) throw ApiError(GBBA_ERR_INVALID_ARGUMENT, "batch handle is NULL");
    if (precision != GBBA_PRECISION_FP64 && precision != GBBA_PRECISION_MIXED)
      throw ApiError(GBBA_ERR_INVALID_ARGUMENT, "unknown precision");
    if (max_iterations < 1 || pcg_iterations < 1 || !(pcg_tolerance > 0.0))
      throw ApiError(GBBA_ERR_INVALID_ARGUMENT, "iteration counts and tolerance must be positive");
    b->precision = precision;
    b->opts.max_iterations = max_iterations;
    b->opts.pcg_iterations = pcg_iterations;
    b->opts.pcg_tolerance = pcg_tolerance;
    if (use_graph < 0 || use_graph > 2) throw ApiError(GBBA_ERR_INVALID_ARGUMENT, "use_graph must be 0, 1 or 2");
    b->opts.use_graph = use_graph;
    b->opts.autotune = autotune != 0;
  });
}

int gbba_batch_set_linear_solver(gbba_batch_t* b, const char* type) {
  return guarded([&] {
    if (!b) throw ApiError(GBBA_ERR_INVALID_ARGUMENT, "batch handle is NULL");
    need(type, "type");
    const std::string s(type);
    if (s == "DENSE_SCHUR" || s == "DENSE_QR" || s == "DENSE_NORMAL_CHOLESKY" || s == "SPARSE_SCHUR" ||
        s == "SPARSE_NORMAL_CHOLESKY")
      b->exact = true;
    else if (s == "ITERATIVE_SCHUR" || s == "CGNR")
      b->exact = false;
    else
      throw ApiError(GBBA_ERR_INVALID_ARGUMENT, "Linear solver type " + s + " doesn't exist.");
  });
}

int gbba_batch_set_function_tolerance(gbba_batch_t* b, double tolerance) {
  return guarded([&] {
    if (!b) throw ApiError(GBBA_ERR_INVALID_ARGUMENT, "batch handle is NULL");
    if (!(tolerance >= 0.0)) throw ApiError(GBBA_ERR_INVALID_ARGUMENT, "tolerance must be non-negative");
    b->opts.function_tolerance = tolerance;
  });
}

int gbba_batch_run(gbba_batch_t* b) {
  return guarded([&] {
    if (!b) throw ApiError(GBBA_ERR_INVALID_ARGUMENT, "batch handle is NULL");
    if (b->items.empty()) throw ApiError(GBBA_ERR_INVALID_ARGUMENT, "batch is empty");
    std::vector<gbba::Problem*> problems;
    // the scale blocks a run set-up adds (relative motions, which batches
    // reject) leave the adjusters on every failure
    auto drop = [&] {
      for (gbba_adjuster_t* item : b->items) ba_of(item).DropScaleBlocks();
    };
    try {
      for (size_t i = 0; i < b->items.size(); ++i) {
        gbba::BundleAdjuster& ba = ba_of(b->items[i]);
        ba.PrepareRun();
        const gbba::SolverOptions& o = ba.Options();
        if (i == 0) {
          b->opts.loss = o.loss;
          b->opts.loss_threshold = o.loss_threshold;
        } else if (o.loss != b->opts.loss || o.loss_threshold != b->opts.loss_threshold) {
          throw ApiError(GBBA_ERR_INVALID_ARGUMENT, "every adjuster of a batch needs the same loss function");
        }
        problems.push_back(&ba.MutableProblem());
      }
      // exact steps: FP64 records and PCG to a 1e-10 relative residual,
      // with at least as many iterations as the largest problem has
      // camera-side unknowns (the finite-termination bound of CG)
      gbba::BatchOptions opts = b->opts;
      int precision = b->precision;
      if (b->exact) {
        precision = GBBA_PRECISION_FP64;
        opts.pcg_tolerance = std::min(opts.pcg_tolerance, kBatchExactTolerance);
        for (gbba::Problem* P : problems)
          opts.pcg_iterations = std::max(opts.pcg_iterations, gbba::camera_side_unknowns(*P));
      }
      auto solver = gbba::make_batch_solver(precision);
      try {
        b->summary = solver->solve_batch(problems, opts);
      } catch (const std::invalid_argument& e) {
        throw ApiError(GBBA_ERR_INVALID_ARGUMENT, e.what());
      }
    } catch (...) {
      drop();
      throw;
    }
    drop();
    for (size_t i = 0; i < b->items.size(); ++i) {
      gbba::BatchProblemSummary& p = b->summary.problems[i];
      gbba::SolveSummary s;
      s.initial_cost = p.initial_cost;
      s.final_cost = p.final_cost;
      s.iterations = p.iterations;
      s.successful_steps = p.successful_steps;
      s.unsuccessful_steps = p.unsuccessful_steps;
      s.termination = p.converged ? "CONVERGENCE" : "NO_CONVERGENCE";
      s.usable = std::isfinite(p.final_cost);
      s.seconds = b->summary.seconds;
      s.linear_solver = b->exact ? "DENSE_SCHUR (GPU batched implicit Schur, FP64 PCG to a 1e-10 relative residual)"
                                 : "ITERATIVE_SCHUR (GPU batched implicit Schur, block-Jacobi PCG)";
      ba_of(b->items[i]).SetBatchResult(s, std::move(p.errors));
    }
    b->has_run = true;
  });
}

int gbba_batch_get_summary(const gbba_batch_t* b, gbba_batch_summary_t* out) {
  return guarded([&] {
    if (!b || !out) throw ApiError(GBBA_ERR_INVALID_ARGUMENT, "NULL argument");
    if (!b->has_run) throw ApiError(GBBA_ERR_RUNTIME, "the batch has not run");
    const gbba::BatchSummary& s = b->summary;
    out->seconds = s.seconds;
    out->setup_seconds = s.setup_seconds;
    out->solve_seconds = s.solve_seconds;
    out->lm_iterations = s.lm_iterations;
    out->grid = s.grid;
    out->n_problems = int(s.problems.size());
    int conv = 0;
    for (const auto& p : s.problems) conv += p.converged ? 1 : 0;
    out->n_converged = conv;
    out->graph_nodes = s.graph_nodes;
    out->kernel_launches = s.kernel_launches;
    out->graph_launches = s.graph_launches;
  });
}

}  // extern "C"
