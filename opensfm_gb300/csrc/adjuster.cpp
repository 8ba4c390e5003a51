#include "adjuster.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <limits>
#include <map>
#include <sstream>
#include <stdexcept>
#include <tuple>

#include "camera_models.cuh"
#include "solver.h"

namespace gbba {

std::vector<int> camera_parameter_types(int model) {
  switch (model) {
    case kPerspective: return {kParamK1, kParamK2, kParamFocal};
    case kBrown:
      return {kParamK1, kParamK2, kParamK3, kParamP1, kParamP2, kParamFocal, kParamAspectRatio, kParamCx, kParamCy};
    case kFisheye: return {kParamK1, kParamK2, kParamFocal};
    case kFisheyeOpencv:
      return {kParamK1, kParamK2, kParamK3, kParamK4, kParamFocal, kParamAspectRatio, kParamCx, kParamCy};
    case kFisheye62:
      return {kParamK1, kParamK2, kParamK3, kParamK4, kParamK5, kParamK6, kParamP1, kParamP2,
              kParamFocal, kParamAspectRatio, kParamCx, kParamCy};
    case kFisheye624:
      return {kParamK1, kParamK2, kParamK3, kParamK4, kParamK5, kParamK6, kParamP1, kParamP2,
              kParamS0, kParamS1, kParamS2, kParamS3, kParamFocal, kParamAspectRatio, kParamCx, kParamCy};
    case kSpherical: return {kParamNone};
    case kDual: return {kParamTransition, kParamK1, kParamK2, kParamFocal};
    case kRadial: return {kParamK1, kParamK2, kParamFocal, kParamAspectRatio, kParamCx, kParamCy};
    case kSimpleRadial: return {kParamK1, kParamFocal, kParamAspectRatio, kParamCx, kParamCy};
  }
  throw std::runtime_error("Invalid ProjectionType");
}

BundleAdjuster::BundleAdjuster() {
  // bundle_adjuster.cc:56-75
  opts_.max_iterations = 500;
  opts_.linear_solver = "SPARSE_SCHUR";
  opts_.loss = kLossTrivial;
  opts_.irls = kIrlsMixture;
  opts_.default_density_ratio = 0.001;
}

// Prior standard deviations of a camera (GetDefaultCameraSigma,
// bundle_adjuster.cc:77-98): parameters without a configured deviation get 0,
// which the prior turns into a weight of 1/epsilon.
void BundleAdjuster::camera_sigma(CameraBlock& c) const {
  const std::vector<int> types = camera_parameter_types(c.model);
  for (int k = 0; k < c.n; ++k) {
    double sd = 0.0;
    switch (types[k]) {
      case kParamFocal: sd = focal_sd_; break;
      case kParamAspectRatio: sd = aspect_sd_; break;
      case kParamCx:
      case kParamCy: sd = c_sd_; break;
      case kParamK1: sd = k1_sd_; break;
      case kParamK2: sd = k2_sd_; break;
      case kParamK3: sd = k3_sd_; break;
      case kParamP1: sd = p1_sd_; break;
      case kParamP2: sd = p2_sd_; break;
      case kParamTransition: sd = 1.0; break;
      default: sd = 0.0;
    }
    c.sigma[k] = sd;
    c.log_prior[k] = (types[k] == kParamFocal || types[k] == kParamAspectRatio) ? 1 : 0;
  }
}

void BundleAdjuster::AddCamera(const std::string& id, int model, const double* values, const double* prior, int n,
                               bool constant) {
  if (model < 0 || model >= kNumProjections) throw std::runtime_error("Invalid ProjectionType");
  if (n != model_num_params(model))
    throw std::invalid_argument("camera " + id + ": expected " + std::to_string(model_num_params(model)) +
                                " parameters, got " + std::to_string(n));
  if (camera_index_.count(id)) return;  // std::map::emplace keeps the first
  CameraBlock c;
  c.model = model;
  c.n = n;
  for (int k = 0; k < n; ++k) {
    c.value[k] = values[k];
    c.prior[k] = prior[k];
    c.free_mask[k] = constant ? 0 : 1;
  }
  camera_index_[id] = int(problem_.cameras.size());
  problem_.cameras.push_back(c);
  problem_.biases.push_back(Bias{});
}

void BundleAdjuster::SetCameraBias(const std::string& camera, const double* rotation, const double* translation,
                                   double scale) {
  auto it = camera_index_.find(camera);
  if (it == camera_index_.end()) throw std::runtime_error("Camera " + camera + " doesn't exist.");
  Bias& b = problem_.biases[it->second];
  for (int k = 0; k < 3; ++k) {
    b.r[k] = rotation[k];
    b.t[k] = translation[k];
  }
  b.s = scale;
}

void BundleAdjuster::SetCameraBiasParameters(const std::string& camera, const int* indices, int n) {
  auto it = camera_index_.find(camera);
  if (it == camera_index_.end()) throw std::runtime_error("Camera " + camera + " doesn't exist.");
  uint8_t mask[7] = {0, 0, 0, 0, 0, 0, 0};
  for (int i = 0; i < n; ++i) {
    if (indices[i] < 0 || indices[i] > 6) throw std::invalid_argument("bias parameter index out of range [0, 6]");
    mask[indices[i]] = 1;
  }
  Bias& b = problem_.biases[it->second];
  for (int k = 0; k < 7; ++k) b.free_mask[k] = mask[k];
}

void BundleAdjuster::GetBias(const std::string& camera, double* rotation, double* translation, double* scale) const {
  auto it = camera_index_.find(camera);
  if (it == camera_index_.end()) throw std::runtime_error("Camera " + camera + " doesn't exist.");
  const Bias& b = problem_.biases[it->second];
  for (int k = 0; k < 3; ++k) {
    rotation[k] = b.r[k];
    translation[k] = b.t[k];
  }
  *scale = b.s;
}

void BundleAdjuster::AddRigCamera(const std::string& id, const double* pose, const double* prior, bool fixed) {
  if (rig_camera_index_.count(id)) throw std::runtime_error("Rig model " + id + " already exist.");
  PoseBlock b;
  for (int k = 0; k < 6; ++k) {
    b.value[k] = pose[k];
    b.prior[k] = prior[k];
    b.free_mask[k] = fixed ? 0 : 1;
  }
  b.has_prior = true;
  rig_camera_index_[id] = int(problem_.rig_cameras.size());
  problem_.rig_cameras.push_back(b);
}

void BundleAdjuster::AddRigInstance(const std::string& id, const double* pose, const std::vector<std::string>& shots,
                                    const std::vector<std::string>& cameras,
                                    const std::vector<std::string>& rig_cameras, bool fixed) {
  int inst;
  auto it = instance_index_.find(id);
  if (it == instance_index_.end()) {
    PoseBlock b;
    for (int k = 0; k < 6; ++k) {
      b.value[k] = pose[k];
      b.free_mask[k] = fixed ? 0 : 1;
    }
    inst = int(problem_.instances.size());
    instance_index_[id] = inst;
    problem_.instances.push_back(b);
  } else {
    inst = it->second;
  }
  for (size_t i = 0; i < shots.size(); ++i) {
    auto c = camera_index_.find(cameras[i]);
    if (c == camera_index_.end()) throw std::runtime_error("Camera " + cameras[i] + " doesn't exist.");
    auto r = rig_camera_index_.find(rig_cameras[i]);
    if (r == rig_camera_index_.end()) throw std::runtime_error("Rig camera " + rig_cameras[i] + " doesn't exist.");
    if (shot_index_.count(shots[i])) continue;
    Shot s;
    s.instance = inst;
    s.camera = c->second;
    s.rig_camera = r->second;
    shot_index_[shots[i]] = int(problem_.shots.size());
    shot_ids_.push_back(shots[i]);
    problem_.shots.push_back(s);
    if (problem_.instances[inst].bias_camera < 0) problem_.instances[inst].bias_camera = c->second;
  }
}

void BundleAdjuster::AddRigInstancePositionPrior(const std::string& id, const double* position,
                                                 const double* std_dev, const std::string& scale_group) {
  auto it = instance_index_.find(id);
  if (it == instance_index_.end()) throw std::runtime_error("Rig instance " + id + " doesn't exist.");
  PoseBlock& b = problem_.instances[it->second];
  b.has_position_prior = true;
  for (int k = 0; k < 3; ++k) {
    b.position_prior[k] = position[k];
    b.position_sigma[k] = std_dev[k];
  }
  int g = -1;
  for (size_t i = 0; i < scale_groups_.size(); ++i)
    if (scale_groups_[i] == scale_group) g = int(i);
  if (g < 0) {
    g = int(scale_groups_.size());
    scale_groups_.push_back(scale_group);
  }
  b.scale_group = g;
}

int64_t BundleAdjuster::AddPoint(const std::string& id, const double* p, bool constant) {
  auto it = point_index_.find(id);
  if (it != point_index_.end()) return it->second;
  PointBlock b;
  for (int k = 0; k < 3; ++k) b.value[k] = p[k];
  b.free = !constant;
  const int64_t idx = int64_t(problem_.points.size());
  point_index_[id] = idx;
  problem_.points.push_back(b);
  return idx;
}

void BundleAdjuster::AddPointPrior(const std::string& id, const double* p, const double* std_dev, bool has_altitude) {
  auto it = point_index_.find(id);
  if (it == point_index_.end()) throw std::runtime_error("Point " + id + " doesn't exist.");
  PointBlock& b = problem_.points[it->second];
  b.has_prior = true;
  for (int k = 0; k < 3; ++k) {
    b.prior[k] = p[k];
    b.sigma[k] = std_dev[k];
  }
  b.has_altitude = has_altitude;
}

void BundleAdjuster::AddPointProjectionObservation(const std::string& shot, const std::string& point,
                                                   const double* obs, double std_dev, bool is_gcp) {
  auto s = shot_index_.find(shot);
  if (s == shot_index_.end()) throw std::out_of_range("map::at: unknown shot " + shot);
  auto p = point_index_.find(point);
  if (p == point_index_.end()) throw std::out_of_range("map::at: unknown point " + point);
  Observation o;
  o.shot = s->second;
  o.point = int(p->second);
  o.x = obs[0];
  o.y = obs[1];
  o.std_dev = std_dev;
  o.is_gcp = is_gcp;
  problem_.observations.push_back(o);
}

void BundleAdjuster::SetObservationDepthPrior(int64_t index, double value, double std_dev, bool is_radial) {
  if (index < 0 || index >= int64_t(problem_.observations.size()))
    throw std::out_of_range("depth prior references an unknown observation");
  if (!(std_dev > 0.0)) throw std::invalid_argument("depth prior std deviation must be positive");
  Observation& o = problem_.observations[size_t(index)];
  o.has_depth = true;
  o.depth_radial = is_radial;
  o.depth = float(value);
  o.depth_std = float(std_dev);
}

int64_t BundleAdjuster::ShotIndex(const std::string& shot) const {
  auto s = shot_index_.find(shot);
  return s == shot_index_.end() ? -1 : s->second;
}

int64_t BundleAdjuster::PointIndex(const std::string& point) const {
  auto p = point_index_.find(point);
  return p == point_index_.end() ? -1 : p->second;
}

int64_t BundleAdjuster::AddPointsBulk(int64_t n, const double* xyz, const uint8_t* constant, const char* const* ids) {
  const int64_t first = int64_t(problem_.points.size());
  problem_.points.reserve(problem_.points.size() + n);
  for (int64_t i = 0; i < n; ++i) {
    const std::string id = ids ? std::string(ids[i]) : std::to_string(first + i);
    if (point_index_.count(id)) throw std::runtime_error("Point " + id + " already exists.");
    PointBlock b;
    for (int k = 0; k < 3; ++k) b.value[k] = xyz[3 * i + k];
    b.free = constant ? constant[i] == 0 : true;
    point_index_[id] = int64_t(problem_.points.size());
    problem_.points.push_back(b);
  }
  return first;
}

void BundleAdjuster::AddObservationsBulk(int64_t n, const int32_t* shot, const int32_t* point, const double* xy,
                                         const double* std_dev, const uint8_t* is_gcp) {
  const int64_t ns = int64_t(problem_.shots.size()), np = int64_t(problem_.points.size());
  for (int64_t i = 0; i < n; ++i) {
    if (shot[i] < 0 || shot[i] >= ns) throw std::out_of_range("observation references an unknown shot");
    if (point[i] < 0 || point[i] >= np) throw std::out_of_range("observation references an unknown point");
    if (!(std_dev[i] > 0.0)) throw std::invalid_argument("observation std deviation must be positive");
  }
  problem_.observations.reserve(problem_.observations.size() + n);
  for (int64_t i = 0; i < n; ++i) {
    Observation o;
    o.shot = shot[i];
    o.point = point[i];
    o.x = xy[2 * i];
    o.y = xy[2 * i + 1];
    o.std_dev = std_dev[i];
    o.is_gcp = is_gcp ? is_gcp[i] != 0 : false;
    problem_.observations.push_back(o);
  }
}

void BundleAdjuster::SetPointProjectionLossFunction(const std::string& name, double threshold) {
  // CreateLossFunction, bundle_adjuster.cc:485-499
  int loss;
  if (name == "TrivialLoss") loss = kLossTrivial;
  else if (name == "HuberLoss") loss = kLossHuber;
  else if (name == "SoftLOneLoss") loss = kLossSoftLOne;
  else if (name == "CauchyLoss") loss = kLossCauchy;
  else if (name == "ArctanLoss") loss = kLossArctan;
  else throw std::runtime_error("ceres::LossFunction with name " + name + " not found.");
  opts_.loss = loss;
  opts_.loss_threshold = threshold;
  loss_name_ = name;
}

void BundleAdjuster::SetInternalParametersPriorSD(double focal, double aspect, double c, double k1, double k2,
                                                  double p1, double p2, double k3, double k4) {
  focal_sd_ = focal;
  aspect_sd_ = aspect;
  c_sd_ = c;
  k1_sd_ = k1;
  k2_sd_ = k2;
  p1_sd_ = p1;
  p2_sd_ = p2;
  k3_sd_ = k3;
  k4_sd_ = k4;
}

void BundleAdjuster::SetRigParametersPriorSD(double translation, double rotation) {
  rig_translation_sd_ = translation;
  rig_rotation_sd_ = rotation;
}

double BundleAdjuster::GetGroupDensityRatio(const std::string& g) const {
  auto it = group_ratio_.find(g);
  return it == group_ratio_.end() ? opts_.default_density_ratio : it->second;
}

void BundleAdjuster::SetShard(int rank, int world, int (*allreduce)(void*, double*, int64_t, int), void* ctx) {
  if (world < 1 || rank < 0 || rank >= world)
    throw std::invalid_argument("shard: rank must be in [0, world_size) and world_size >= 1");
  if (world > 1 && !allreduce) throw std::invalid_argument("shard: a world_size above 1 needs an all-reduce");
  opts_.shard.rank = rank;
  opts_.shard.world = world;
  opts_.shard.allreduce = world > 1 ? allreduce : nullptr;
  opts_.shard.ctx = world > 1 ? ctx : nullptr;
}

std::pair<int64_t, int64_t> BundleAdjuster::ShardRange(int rank) const {
  const int64_t np = int64_t(problem_.points.size());
  const int world = std::max(1, opts_.shard.world);
  if (world == 1) return {0, np};
  if (rank < 0 || rank >= world) throw std::invalid_argument("shard: rank out of range");
  // rank r starts at the first point before which at least r/world of the
  // observations lie
  std::vector<int64_t> cum(size_t(np) + 1, 0);
  for (const Observation& o : problem_.observations) ++cum[size_t(o.point) + 1];
  for (int64_t p = 0; p < np; ++p) cum[size_t(p) + 1] += cum[size_t(p)];
  const int64_t total = cum[size_t(np)];
  auto start = [&](int r) -> int64_t {
    if (r <= 0) return 0;
    if (r >= world) return np;
    const int64_t want = (total * r + world - 1) / world;  // ceil(total r / world)
    return int64_t(std::lower_bound(cum.begin(), cum.end(), want) - cum.begin());
  };
  const int64_t a = std::min(start(rank), np), b = std::min(std::max(start(rank + 1), a), np);
  return {a, b};
}

CoarseSpace BundleAdjuster::CoarseLayout(int leaf) {
  PrepareRun();
  std::vector<uint8_t> fm(problem_.instances.size() * 6);
  for (size_t i = 0; i < problem_.instances.size(); ++i)
    for (int k = 0; k < 6; ++k) fm[6 * i + k] = problem_.instances[i].free_mask[k];
  return build_coarse_space(problem_, fm, leaf, point_major_order(problem_));
}

void BundleAdjuster::Run() {
  PrepareRun();
  opts_.compute_covariances = compute_covariances_;
  const bool shard = opts_.shard.active();
  // Sharded: the problem without points and observations, then this
  // rank's points and the observations of them (point indices relative to
  // the range's first point).
  Problem sub;
  std::vector<int64_t> sub_obs;  // index in problem_.observations of each of sub's observations
  int64_t p0 = 0, p1 = 0;
  if (shard) {
    std::tie(p0, p1) = ShardRange(opts_.shard.rank);
    std::vector<PointBlock> pts;
    std::vector<Observation> obs;
    pts.swap(problem_.points);
    obs.swap(problem_.observations);
    sub = problem_;
    pts.swap(problem_.points);
    obs.swap(problem_.observations);
    sub.points.assign(problem_.points.begin() + p0, problem_.points.begin() + p1);
    for (size_t i = 0; i < problem_.observations.size(); ++i) {
      const Observation& o = problem_.observations[i];
      if (o.point < p0 || o.point >= p1) continue;
      Observation q = o;
      q.point = int(o.point - p0);
      sub.observations.push_back(q);
      sub_obs.push_back(int64_t(i));
    }
    opts_.compute_covariances = false;
  }
  // Mixed precision is for the iterative path.  Exact dense steps solve the
  // explicit reduced camera system, whose assembly is FP64 in both
  // precisions; FP32 Jacobians there only perturb the gauge directions of
  // S (nearly singular without a gauge prior), which the exact solve then
  // amplifies into rejected steps.  Such runs take FP64 records.
  const bool exact = exact_dense_steps(shard ? sub : problem_, opts_);
  const int precision = exact ? 0 : opts_.precision;
  std::unique_ptr<SolverBase> solver;
  try {
    solver = make_solver(precision);
    summary_ = solver->solve(shard ? sub : problem_, opts_);
    if (exact && opts_.precision != 0) summary_.linear_solver += "; FP64 records (exact steps)";
  } catch (...) {
    DropScaleBlocks();
    throw;
  }
  if (shard) {
    // the camera side (identical on every rank) and this rank's points
    for (size_t c = 0; c < sub.cameras.size(); ++c) problem_.cameras[c] = sub.cameras[c];
    for (size_t r = 0; r < sub.rig_cameras.size(); ++r) problem_.rig_cameras[r] = sub.rig_cameras[r];
    for (size_t i = 0; i < sub.instances.size(); ++i) problem_.instances[i] = sub.instances[i];
    for (int64_t p = p0; p < p1; ++p) problem_.points[size_t(p)] = sub.points[size_t(p - p0)];
  }
  // the solved reconstruction scales and camera biases, then the rig
  // cameras without the scale blocks again
  for (const ScaleBlock& b : scale_blocks_) {
    if (b.reconstruction_scale)
      reconstructions_.at(b.reconstruction).scales[b.instance] = problem_.rig_cameras[b.block].value[0];
    if (b.bias_camera >= 0) {
      Bias& bs = problem_.biases[size_t(b.bias_camera)];
      const PoseBlock& pose = problem_.rig_cameras[size_t(b.block)];
      for (int k = 0; k < 3; ++k) {
        bs.r[k] = pose.value[k];
        bs.t[k] = pose.value[3 + k];
      }
      bs.s = problem_.rig_cameras[size_t(b.block) + 1].value[0];
    }
  }
  DropScaleBlocks();
  if (opts_.compute_reprojection_errors && shard) {
    // this rank's observations; the others' are NaN here
    std::vector<double> e, w;
    solver->reprojection(e, w);
    errors_.assign(3 * problem_.observations.size(), std::numeric_limits<double>::quiet_NaN());
    weights_.assign(problem_.observations.size(), std::numeric_limits<double>::quiet_NaN());
    for (size_t k = 0; k < sub_obs.size(); ++k) {
      const size_t i = size_t(sub_obs[k]);
      for (int a = 0; a < 3; ++a) errors_[3 * i + a] = e[3 * k + a];
      weights_[i] = w[k];
    }
  } else if (opts_.compute_reprojection_errors) {
    solver->reprojection(errors_, weights_);
  } else {
    errors_.clear();
    weights_.clear();
  }
  covariance_valid_ = false;
  covariances_.clear();
  if (compute_covariances_) {
    std::vector<double> cov;
    covariance_valid_ = summary_.termination != "FAILURE" && solver->covariances(cov) &&
                        cov.size() == 36 * problem_.instances.size();
    if (covariance_valid_) {
      covariances_ = std::move(cov);
    } else {
      // the reference's fallback (bundle_adjuster.cc:1272-1286)
      covariances_.assign(36 * problem_.instances.size(), 0.0);
      for (size_t i = 0; i < problem_.instances.size(); ++i)
        for (int k = 0; k < 6; ++k) covariances_[36 * i + 7 * k] = k < 3 ? 1e-5 : 1e-2;
    }
  }
  has_run_ = true;
}

void BundleAdjuster::GetRigInstanceCovariance(const std::string& id, double* out) const {
  const auto it = instance_index_.find(id);
  if (it == instance_index_.end()) throw std::runtime_error("Rig instance " + id + " doesn't exist.");
  if (covariances_.empty()) throw std::runtime_error("no covariance: run with set_compute_covariances(true)");
  for (int k = 0; k < 36; ++k) out[k] = covariances_[36 * size_t(it->second) + k];
}

void BundleAdjuster::SetBatchResult(const SolveSummary& s, std::vector<double> errors) {
  summary_ = s;
  if (opts_.compute_reprojection_errors) {
    errors_ = std::move(errors);
    weights_.assign(problem_.observations.size(), 1.0);
  } else {
    errors_.clear();
    weights_.clear();
  }
  covariance_valid_ = false;
  has_run_ = true;
}

void BundleAdjuster::AddOrientationConstraint(const std::string& shot_id, int kind, const double* value,
                                              double std_deviation) {
  if (kind < OrientationTerm::kUpVector || kind > OrientationTerm::kRoll)
    throw std::invalid_argument("unknown orientation constraint kind");
  if (shot_index_.find(shot_id) == shot_index_.end()) throw std::out_of_range("Shot " + shot_id + " doesn't exist.");
  PendingOrientation o{shot_id, kind, {value[0], kind == OrientationTerm::kUpVector ? value[1] : 0.0,
                                      kind == OrientationTerm::kUpVector ? value[2] : 0.0},
                       std_deviation};
  orientations_.push_back(o);
}

void BundleAdjuster::AddRelativeRotation(const std::string& shot_i, const std::string& shot_j,
                                         const double* rotation, const double* scale_matrix) {
  PendingRelative r{};
  r.kind = RelativeTerm::kRelativeRotation;
  r.shots[0] = shot_i;
  r.shots[1] = shot_j;
  for (int k = 0; k < 3; ++k) r.rotation[k] = rotation[k];
  for (int k = 0; k < 9; ++k) r.scale_matrix[k] = scale_matrix ? scale_matrix[k] : (k % 4 == 0 ? 1.0 : 0.0);
  for (int k = 0; k < 2; ++k)
    if (shot_index_.find(r.shots[k]) == shot_index_.end())
      throw std::out_of_range("Shot " + r.shots[k] + " doesn't exist.");
  relatives_.push_back(r);
}

void BundleAdjuster::AddCommonPosition(const std::string& shot_i, const std::string& shot_j, double margin,
                                       double std_deviation) {
  PendingRelative r{};
  r.kind = RelativeTerm::kCommonPosition;
  r.shots[0] = shot_i;
  r.shots[1] = shot_j;
  r.margin = margin;
  r.std_deviation = std_deviation;
  for (int k = 0; k < 2; ++k)
    if (shot_index_.find(r.shots[k]) == shot_index_.end())
      throw std::out_of_range("Shot " + r.shots[k] + " doesn't exist.");
  relatives_.push_back(r);
}

void BundleAdjuster::AddLinearMotion(const std::string& shot0, const std::string& shot1, const std::string& shot2,
                                     double alpha, double position_std_deviation, double orientation_std_deviation) {
  PendingRelative r{};
  r.kind = RelativeTerm::kLinearMotion;
  r.shots[0] = shot0;
  r.shots[1] = shot1;
  r.shots[2] = shot2;
  r.alpha = alpha;
  r.position_std = position_std_deviation;
  r.orientation_std = orientation_std_deviation;
  for (int k = 0; k < 3; ++k)
    if (shot_index_.find(r.shots[k]) == shot_index_.end())
      throw std::out_of_range("Shot " + r.shots[k] + " doesn't exist.");
  relatives_.push_back(r);
}

void BundleAdjuster::SetRelativeMotionLossFunction(const std::string& name, double threshold) {
  relative_loss_name_ = name;
  relative_loss_threshold_ = threshold;
}

void BundleAdjuster::SetGaugeFixShots(const std::string& shot_origin, const std::string& shot_scale) {
  const auto it = shot_index_.find(shot_origin);
  if (it == shot_index_.end()) throw std::out_of_range("Shot " + shot_origin + " doesn't exist.");
  PoseBlock& inst = problem_.instances[problem_.shots[it->second].instance];
  for (int k = 0; k < 6; ++k) inst.free_mask[k] = 0;
  has_gauge_ = true;
  gauge_shots_[0] = shot_origin;
  gauge_shots_[1] = shot_scale;
}

void BundleAdjuster::AddHeatmap(const std::string& id, const double* data, int64_t n, int64_t width,
                                double resolution) {
  if (width <= 0 || n < width || n % width != 0)
    throw std::invalid_argument("heatmap " + id + ": size must be a positive multiple of the width");
  Problem::Heatmap h;
  h.data.assign(data, data + n);
  h.width = int(width);
  h.resolution = resolution;
  const auto it = heatmap_index_.find(id);
  if (it != heatmap_index_.end()) {
    problem_.heatmaps[it->second] = std::move(h);  // the reference replaces the grid of an id
  } else {
    heatmap_index_[id] = int(problem_.heatmaps.size());
    problem_.heatmaps.push_back(std::move(h));
  }
}

void BundleAdjuster::AddAbsolutePositionHeatmap(const std::string& shot, const std::string& heatmap_id,
                                                double x_offset, double y_offset, double std_deviation) {
  if (shot_index_.find(shot) == shot_index_.end()) throw std::out_of_range("Shot " + shot + " doesn't exist.");
  const auto it = heatmap_index_.find(heatmap_id);
  if (it == heatmap_index_.end()) throw std::out_of_range("Heatmap " + heatmap_id + " doesn't exist.");
  heatmap_terms_.push_back({shot, it->second, x_offset, y_offset, std_deviation});
}

void BundleAdjuster::AddReconstruction(const std::string& id, bool constant) {
  ReconstructionScales r;
  r.constant = constant;
  r.shared = true;
  reconstructions_[id] = r;
}

void BundleAdjuster::AddReconstructionInstance(const std::string& reconstruction_id, double scale,
                                               const std::string& instance_id) {
  const auto it = reconstructions_.find(reconstruction_id);
  if (it == reconstructions_.end()) return;
  it->second.scales[instance_id] = scale;
  reconstruction_of_[instance_id] = reconstruction_id;
}

void BundleAdjuster::SetScaleSharing(const std::string& id, bool share) {
  const auto it = reconstructions_.find(id);
  if (it != reconstructions_.end()) it->second.shared = share;
}

double BundleAdjuster::GetReconstructionScale(const std::string& reconstruction_id,
                                              const std::string& instance_id) const {
  const auto it = reconstructions_.find(reconstruction_id);
  if (it == reconstructions_.end())
    throw std::runtime_error("Reconstruction " + reconstruction_id + " doesn't exist.");
  const ReconstructionScales& r = it->second;
  if (r.shared) {
    if (r.scales.empty()) throw std::out_of_range("Reconstruction " + reconstruction_id + " has no instance.");
    return r.scales.begin()->second;
  }
  return r.scales.at(instance_id);
}

void BundleAdjuster::AddRelativeMotion(const std::string& instance_i, const std::string& instance_j,
                                       const double* motion, double robust_multiplier, bool observed_scale,
                                       const double* scale_matrix) {
  PendingMotion m{};
  m.instances[0] = instance_i;
  m.instances[1] = instance_j;
  for (int k = 0; k < 7; ++k) m.motion[k] = motion[k];
  for (int k = 0; k < 49; ++k) m.scale_matrix[k] = scale_matrix ? scale_matrix[k] : (k % 8 == 0 ? 1.0 : 0.0);
  m.robust_multiplier = robust_multiplier;
  m.observed_scale = observed_scale;
  motions_.push_back(m);
}

void BundleAdjuster::DropScaleBlocks() {
  for (int i : moved_priors_) problem_.instances[i].has_position_prior = true;
  moved_priors_.clear();
  if (scale_blocks_.empty()) return;
  problem_.rig_cameras.resize(n_rig_cameras_);
  scale_blocks_.clear();
}

void BundleAdjuster::PrepareRun() {
  DropScaleBlocks();
  static const char* kSolvers[] = {"DENSE_NORMAL_CHOLESKY", "DENSE_QR", "SPARSE_NORMAL_CHOLESKY", "DENSE_SCHUR",
                                   "SPARSE_SCHUR", "ITERATIVE_SCHUR", "CGNR"};
  bool known = false;
  for (const char* s : kSolvers) known |= opts_.linear_solver == s;
  if (!known) throw std::runtime_error("Linear solver type " + opts_.linear_solver + " doesn't exist.");
  problem_.orientation_terms.clear();
  for (const PendingOrientation& o : orientations_) {
    if (!(o.std_deviation > 0.0)) continue;
    const Shot& sh = problem_.shots[shot_index_.at(o.shot)];
    OrientationTerm t;
    t.kind = o.kind;
    t.instance = sh.instance;
    t.rig_camera = sh.rig_camera;
    t.scale = 1.0 / o.std_deviation;
    if (o.kind == OrientationTerm::kUpVector) {
      // UpVectorError normalizes the direction (absolute_motion_errors.h:11-14)
      const double n = std::sqrt(o.value[0] * o.value[0] + o.value[1] * o.value[1] + o.value[2] * o.value[2]);
      for (int k = 0; k < 3; ++k) t.target[k] = n > 0.0 ? o.value[k] / n : 0.0;
    } else {
      t.target[0] = o.value[0];
    }
    problem_.orientation_terms.push_back(t);
  }
  // sigmas and usage flags at run time
  for (CameraBlock& c : problem_.cameras) camera_sigma(c);
  for (PoseBlock& r : problem_.rig_cameras) {
    for (int k = 0; k < 3; ++k) {
      r.sigma[k] = rig_rotation_sd_;
      r.sigma[3 + k] = rig_translation_sd_;
    }
    bool any_free = false, all_zero = true;
    for (int k = 0; k < 6; ++k) {
      any_free |= r.free_mask[k] != 0;
      all_zero &= r.value[k] == 0.0;
    }
    r.used = !(!any_free && all_zero);  // IsRigCameraUseful, bundle_adjuster.cc:20-23
  }
  // IRLS density ratios: defaults, then per-group overrides
  problem_.group_density_ratio.assign(problem_.shots.size() + 1, opts_.default_density_ratio);
  for (size_t s = 0; s < shot_ids_.size(); ++s) problem_.group_density_ratio[s] = GetGroupDensityRatio("PROJ_" + shot_ids_[s]);
  problem_.group_density_ratio[shot_ids_.size()] = GetGroupDensityRatio("GCP2D");
  problem_.ratio_cam = GetGroupDensityRatio("CAM");
  problem_.ratio_rig = GetGroupDensityRatio("RCAM");
  problem_.ratio_gps = GetGroupDensityRatio("GPS");
  problem_.ratio_gcp3d = GetGroupDensityRatio("GCP3D");
  problem_.ratio_depth = GetGroupDensityRatio("DEPTH");
  // AddRelativeDepthError refuses a non-finite depth (bundle_adjuster.cc:582-586)
  for (const Observation& o : problem_.observations)
    if (o.has_depth && !std::isfinite(o.depth))
      throw std::runtime_error(shot_ids_[size_t(o.shot)] + " has non-finite depth prior");
  static const char* kHostGroups[12] = {"UP",     "PAN",   "TILT",    "ROLL", "ROT", "POS",
                                        "MOTION", "GAUGE", "HEATMAP", "REL",  "GPS", "STDDEV"};
  for (int k = 0; k < 12; ++k) problem_.ratio_host[k] = GetGroupDensityRatio(kHostGroups[k]);
  // constraints between shots, composed with the rig cameras that are
  // optimised or not the identity (IsRigCameraUseful), as Run passes them
  // (bundle_adjuster.cc:912-1138)
  problem_.relative_terms.clear();
  bool any_rotation = false;
  for (const PendingRelative& p : relatives_) {
    RelativeTerm t;
    t.kind = p.kind;
    t.n_shots = p.kind == RelativeTerm::kLinearMotion ? 3 : 2;
    int rc[3] = {-1, -1, -1};
    for (int k = 0; k < t.n_shots; ++k) {
      const Shot& sh = problem_.shots[shot_index_.at(p.shots[k])];
      t.instance[k] = sh.instance;
      rc[k] = sh.rig_camera >= 0 && problem_.rig_cameras[sh.rig_camera].used ? sh.rig_camera : -1;
      t.rig_camera[k] = rc[k];
    }
    if (p.kind == RelativeTerm::kLinearMotion && rc[2] >= 0 && (rc[2] == rc[0] || rc[2] == rc[1]))
      t.rig_camera[2] = rc[0];  // LinearMotionError reads shot 0's rig camera then (bundle_adjuster.cc:1124-1134)
    for (int k = 0; k < 3; ++k) t.rotation[k] = p.rotation[k];
    for (int k = 0; k < 9; ++k) t.scale_matrix[k] = p.scale_matrix[k];
    t.margin = p.margin;
    t.scale = 1.0 / p.std_deviation;
    t.alpha = p.alpha;
    t.position_scale = 1.0 / p.position_std;
    t.orientation_scale = 1.0 / p.orientation_std;
    any_rotation |= p.kind == RelativeTerm::kRelativeRotation;
    problem_.relative_terms.push_back(t);
  }
  for (const PendingHeatmap& p : heatmap_terms_) {
    // the shot position always composes the rig camera (the functor gets
    // its parameter block whether or not it is optimised)
    const Shot& sh = problem_.shots[shot_index_.at(p.shot)];
    const Problem::Heatmap& hm = problem_.heatmaps[p.heatmap];
    RelativeTerm t;
    t.kind = RelativeTerm::kHeatmap;
    t.n_shots = 1;
    t.instance[0] = sh.instance;
    t.rig_camera[0] = sh.rig_camera;
    t.grid.data = hm.data.data();
    t.grid.width = hm.width;
    t.grid.height = int(hm.data.size() / size_t(hm.width));
    t.grid.resolution = hm.resolution;
    t.x_offset = p.x_offset;
    t.y_offset = p.y_offset;
    t.scale = 1.0 / p.std_deviation;
    problem_.relative_terms.push_back(t);
  }
  if (has_gauge_) {
    RelativeTerm t;
    t.kind = RelativeTerm::kGaugeScale;
    t.n_shots = 2;
    for (int k = 0; k < 2; ++k) {
      const auto it = shot_index_.find(gauge_shots_[k]);
      if (it == shot_index_.end()) throw std::out_of_range("Shot " + gauge_shots_[k] + " doesn't exist.");
      t.instance[k] = problem_.shots[it->second].instance;
    }
    const double* a = problem_.instances[t.instance[0]].value + 3;
    const double* b = problem_.instances[t.instance[1]].value + 3;
    t.distance = std::sqrt((a[0] - b[0]) * (a[0] - b[0]) + (a[1] - b[1]) * (a[1] - b[1]) + (a[2] - b[2]) * (a[2] - b[2]));
    problem_.relative_terms.push_back(t);
  }
  // relative motions: the reconstruction scales become one-coordinate
  // blocks after the rig cameras (a shared scale is the reconstruction's
  // first entry, as Reconstruction::GetScalePtr picks it)
  n_rig_cameras_ = problem_.rig_cameras.size();
  if (!motions_.empty()) {
    auto block_of = [&](const std::string& instance) {
      const std::string& rec_id = reconstruction_of_.at(instance);
      ReconstructionScales& rec = reconstructions_.at(rec_id);
      const std::string key = rec.shared ? rec.scales.begin()->first : instance;
      for (const ScaleBlock& b : scale_blocks_)
        if (b.reconstruction_scale && b.reconstruction == rec_id && b.instance == key) return b.block;
      PoseBlock pb;
      pb.value[0] = rec.scales.at(key);
      pb.free_mask[0] = rec.constant ? 0 : 1;
      pb.has_prior = false;
      pb.used = true;
      pb.scale_block = true;
      const int block = int(problem_.rig_cameras.size());
      problem_.rig_cameras.push_back(pb);
      scale_blocks_.push_back({rec_id, key, block, true});
      return block;
    };
    try {
      for (const PendingMotion& m : motions_) {
        RelativeTerm t;
        t.kind = RelativeTerm::kRelativeMotion;
        t.n_shots = 2;
        for (int k = 0; k < 2; ++k) {
          const auto it = instance_index_.find(m.instances[k]);
          if (it == instance_index_.end())
            throw std::out_of_range("Rig instance " + m.instances[k] + " doesn't exist.");
          t.instance[k] = it->second;
          t.scale_block[k] = block_of(m.instances[k]);
        }
        for (int k = 0; k < 7; ++k) t.motion[k] = m.motion[k];
        for (int k = 0; k < 49; ++k) t.motion_matrix[k] = m.scale_matrix[k];
        t.observed_scale = m.observed_scale;
        t.loss_scale = relative_loss_threshold_ * m.robust_multiplier;
        problem_.relative_terms.push_back(t);
      }
    } catch (...) {
      DropScaleBlocks();
      throw;
    }
    any_rotation = true;  // the relative-motion loss is needed
  }
  // GPS priors as host terms: every prior when the std multipliers are
  // adjusted (one per scale group, starting at 1, each with a
  // StdDeviationConstraint, bundle_adjuster.cc:772-838), and the priors
  // whose reference camera has an optimised bias (its rotation and
  // translation a six-coordinate block, its scale a one-coordinate block,
  // both after the rig cameras; SimilarityPriorTransform, bias.h:34-54).
  std::map<int, int> group_block;
  std::map<int, int> bias_block;
  auto bias_block_of = [&](int cam) -> int {
    auto it = bias_block.find(cam);
    if (it != bias_block.end()) return it->second;
    const Bias& bs = problem_.biases[size_t(cam)];
    PoseBlock pose, scale;
    for (int k = 0; k < 3; ++k) {
      pose.value[k] = bs.r[k];
      pose.value[3 + k] = bs.t[k];
    }
    for (int k = 0; k < 6; ++k) pose.free_mask[k] = bs.free_mask[k];
    scale.value[0] = bs.s;
    scale.free_mask[0] = bs.free_mask[6];
    for (PoseBlock* b : {&pose, &scale}) {
      b->has_prior = false;
      b->used = true;
      b->scale_block = true;
    }
    const int block = int(problem_.rig_cameras.size());
    problem_.rig_cameras.push_back(pose);
    problem_.rig_cameras.push_back(scale);
    ScaleBlock sb;
    sb.block = block;
    sb.reconstruction_scale = false;
    sb.bias_camera = cam;
    scale_blocks_.push_back(sb);
    bias_block.emplace(cam, block);
    return block;
  };
  // (when some prior takes an optimised bias, every GPS prior becomes a host
  // term, so that they stay one IRLS group "GPS" as in the reference)
  bool any_biased = false;
  for (const PoseBlock& b : problem_.instances)
    any_biased |= b.has_position_prior && b.bias_camera >= 0 && problem_.biases[size_t(b.bias_camera)].optimised();
  for (size_t i = 0; i < problem_.instances.size(); ++i) {
    PoseBlock& b = problem_.instances[i];
    if (!b.has_position_prior) continue;
    const bool biased = b.bias_camera >= 0 && problem_.biases[size_t(b.bias_camera)].optimised();
    if (!adjust_position_std_ && !any_biased) continue;
    RelativeTerm t;
    t.kind = RelativeTerm::kGpsStd;
    t.n_shots = 1;
    t.instance[0] = int(i);
    for (int k = 0; k < 3; ++k) {
      t.prior[k] = b.position_prior[k];
      t.prior_scale[k] = 1.0 / std::max(b.position_sigma[k], std::numeric_limits<double>::epsilon());
    }
    t.bias_camera = b.bias_camera;
    if (biased) {
      t.bias_block[0] = bias_block_of(b.bias_camera);
      t.bias_block[1] = t.bias_block[0] + 1;
    }
    if (adjust_position_std_) {
      auto g = group_block.find(b.scale_group);
      if (g == group_block.end()) {
        PoseBlock pb;
        pb.value[0] = 1.0;
        pb.free_mask[0] = 1;
        pb.has_prior = false;
        pb.used = true;
        pb.scale_block = true;
        const int block = int(problem_.rig_cameras.size());
        problem_.rig_cameras.push_back(pb);
        scale_blocks_.push_back({"", "", block, false});
        g = group_block.emplace(b.scale_group, block).first;
      }
      t.scale_block[0] = g->second;
    }
    problem_.relative_terms.push_back(t);
    b.has_position_prior = false;  // the diagonal GPS prior is replaced
    moved_priors_.push_back(int(i));
  }
  for (const auto& gb : group_block) {
    RelativeTerm t;
    t.kind = RelativeTerm::kStdDeviation;
    t.n_shots = 0;
    t.scale_block[0] = gb.second;
    problem_.relative_terms.push_back(t);
  }
  if (any_rotation) {
    // CreateLossFunction (bundle_adjuster.cc:485-499)
    const std::string& n = relative_loss_name_;
    int loss;
    if (n == "TrivialLoss") loss = kLossTrivial;
    else if (n == "HuberLoss") loss = kLossHuber;
    else if (n == "SoftLOneLoss") loss = kLossSoftLOne;
    else if (n == "CauchyLoss") loss = kLossCauchy;
    else if (n == "ArctanLoss") loss = kLossArctan;
    else {
      DropScaleBlocks();
      throw std::runtime_error("ceres::LossFunction with name " + n + " not found.");
    }
    problem_.relative_loss = loss;
    problem_.relative_loss_threshold = relative_loss_threshold_;
  }
}

int BundleAdjuster::GetCamera(const std::string& id, int* model, double* values, int cap) const {
  auto it = camera_index_.find(id);
  if (it == camera_index_.end()) throw std::runtime_error("Camera " + id + " doesn't exists");
  const CameraBlock& c = problem_.cameras[it->second];
  if (model) *model = c.model;
  for (int k = 0; k < std::min(cap, c.n); ++k) values[k] = c.value[k];
  return c.n;
}

void BundleAdjuster::GetRigInstancePose(const std::string& id, double* pose) const {
  auto it = instance_index_.find(id);
  if (it == instance_index_.end()) throw std::runtime_error("Rig instance " + id + " doesn't exists");
  for (int k = 0; k < 6; ++k) pose[k] = problem_.instances[it->second].value[k];
}

void BundleAdjuster::GetRigCameraPose(const std::string& id, double* pose) const {
  auto it = rig_camera_index_.find(id);
  if (it == rig_camera_index_.end()) throw std::runtime_error("Rig camera " + id + " doesn't exists");
  for (int k = 0; k < 6; ++k) pose[k] = problem_.rig_cameras[it->second].value[k];
}

void BundleAdjuster::GetPoint(const std::string& id, double* p) const {
  auto it = point_index_.find(id);
  if (it == point_index_.end()) throw std::runtime_error("Point " + id + " doesn't exists");
  for (int k = 0; k < 3; ++k) p[k] = problem_.points[it->second].value[k];
}

void BundleAdjuster::GetPointsBulk(int64_t first, int64_t n, double* xyz) const {
  if (first < 0 || first + n > int64_t(problem_.points.size())) throw std::out_of_range("point range");
  for (int64_t i = 0; i < n; ++i)
    for (int k = 0; k < 3; ++k) xyz[3 * i + k] = problem_.points[first + i].value[k];
}

std::vector<int32_t> BundleAdjuster::ObservationPoints() const {
  std::vector<int32_t> out(problem_.observations.size());
  for (size_t i = 0; i < out.size(); ++i) out[i] = int32_t(problem_.observations[i].point);
  return out;
}

void BundleAdjuster::GetProjectionResults(int64_t n, double* errors, double* weights, int32_t* dims) const {
  if (n != int64_t(problem_.observations.size())) throw std::invalid_argument("wrong observation count");
  const bool have = has_run_ && errors_.size() == size_t(3 * n);
  for (int64_t i = 0; i < n; ++i) {
    const Observation& o = problem_.observations[i];
    const int dim = problem_.cameras[problem_.shots[o.shot].camera].model == kSpherical ? 3 : 2;
    if (dims) dims[i] = dim;
    for (int k = 0; k < 3; ++k) errors[3 * i + k] = have ? errors_[3 * i + k] : 0.0;
    if (weights) weights[i] = have ? weights_[i] : 1.0;
  }
}

std::string BundleAdjuster::BriefReport() const {
  char buf[512];
  std::snprintf(buf, sizeof(buf),
                "GB300 Bundle Adjuster Report: Iterations: %d, Initial cost: %e, Final cost: %e, Termination: %s",
                summary_.iterations, summary_.initial_cost, summary_.final_cost, summary_.termination.c_str());
  return buf;
}

std::string BundleAdjuster::FullReport() const {
  std::ostringstream ss;
  ss << "GB300 Bundle Adjuster Report\n";
  ss << "  Precision            " << (opts_.precision == 0 ? "FP64" : "mixed FP32/FP64") << "\n";
  ss << "  Linear solver        " << summary_.linear_solver << "\n";
  ss << "  Loss                 " << loss_name_ << " (threshold " << opts_.loss_threshold << ")\n";
  ss << "  IRLS                 " << (opts_.irls == kIrlsMixture ? "mixture" : "none") << "\n";
  ss << "  Cameras / shots      " << problem_.cameras.size() << " / " << problem_.shots.size() << "\n";
  ss << "  Points / projections " << problem_.points.size() << " / " << problem_.observations.size() << "\n";
  ss << "  Initial cost         " << summary_.initial_cost << "\n";
  ss << "  Final cost           " << summary_.final_cost << "\n";
  ss << "  Iterations           " << summary_.iterations << " (" << summary_.successful_steps << " successful, "
     << summary_.unsuccessful_steps << " unsuccessful)\n";
  ss << "  Time (s)             total " << summary_.seconds << ", linear solver " << summary_.linear_solver_seconds
     << ", jacobian " << summary_.jacobian_seconds << ", residuals " << summary_.residual_seconds << ", setup "
     << summary_.setup_seconds << "\n";
  ss << "  Kernel launches      " << summary_.kernel_launches << "\n";
  ss << "  PCG refinements      " << summary_.pcg_refinements << " (FP64 residuals of the mixed-precision solve)\n";
  ss << "  Dense failures       " << summary_.linear_solver_failures
     << " (factorizations of a damped system that was not positive definite)\n";
  ss << "  Jacobians            " << (summary_.matrix_free ? "matrix-free (evaluated in every pass)" : "stored")
     << "\n";
  ss << "  Termination          " << summary_.termination << "\n";
  return ss.str();
}

std::string BundleAdjuster::IrlsReport() const {
  std::ostringstream ss;
  for (size_t i = 0; i < summary_.irls_lines.size(); ++i) {
    if (i) ss << "\n";
    ss << summary_.irls_lines[i];
  }
  return ss.str();
}

}  // namespace gbba
