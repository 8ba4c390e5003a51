// Host-side bundle adjuster with the reference's API semantics
// (bundle::BundleAdjuster, opensfm/src/lib/bundle/bundle_adjuster.h:173-386,
// src/bundle_adjuster.cc:56-1400): string-keyed cameras, rig cameras, rig
// instances (which create the shots), points and observations; settings;
// Run(); getters and reports.  The optimisation itself runs on the GPU
// (solver.h).
#pragma once

#include <map>
#include <string>
#include <unordered_map>
#include <vector>

#include "coarse_space.h"
#include "problem.h"

namespace gbba {

class BundleAdjuster {
 public:
  BundleAdjuster();

  // adders (bundle_adjuster.cc:107-301)
  void AddCamera(const std::string& id, int model, const double* values, const double* prior, int n, bool constant);
  void AddRigCamera(const std::string& id, const double* pose, const double* prior, bool fixed);
  void AddRigInstance(const std::string& id, const double* pose, const std::vector<std::string>& shots,
                      const std::vector<std::string>& cameras, const std::vector<std::string>& rig_cameras,
                      bool fixed);
  void AddRigInstancePositionPrior(const std::string& id, const double* position, const double* std_dev,
                                   const std::string& scale_group);
  int64_t AddPoint(const std::string& id, const double* p, bool constant);
  void AddPointPrior(const std::string& id, const double* p, const double* std_dev, bool has_altitude);
  // Absolute orientation constraints of a shot (bundle_adjuster.cc:352-395):
  // kind OrientationTerm::kUpVector (value = 3-vector) or kPan / kTilt /
  // kRoll (value[0] = angle).  Constraints with std_deviation <= 0 are kept
  // and ignored, as the reference adds only positive ones.
  void AddOrientationConstraint(const std::string& shot_id, int kind, const double* value, double std_deviation);
  // Constraints between shots (bundle_adjuster.cc:303-320, 503-514): a
  // relative rotation R_ij with a 3 x 3 scale matrix (null: identity), a
  // common position within a horizontal margin, and linear motion of shot1
  // between shot0 and shot2 at fraction alpha.
  void AddRelativeRotation(const std::string& shot_i, const std::string& shot_j, const double* rotation,
                           const double* scale_matrix);
  void AddCommonPosition(const std::string& shot_i, const std::string& shot_j, double margin, double std_deviation);
  void AddLinearMotion(const std::string& shot0, const std::string& shot1, const std::string& shot2, double alpha,
                       double position_std_deviation, double orientation_std_deviation);
  // the loss of the relative rotations (SetRelativeMotionLossFunction,
  // bundle_adjuster.cc:396-400); the name is checked when a run needs it
  void SetRelativeMotionLossFunction(const std::string& name, double threshold);
  // SetGaugeFixShots (bundle_adjuster.cc:389-394): the origin shot's rig
  // instance becomes constant; a run adds log(|t1 - t2| / d) between the
  // two shots' rig instance positions, d their distance at the start of the
  // run (:1140-1157).
  void SetGaugeFixShots(const std::string& shot_origin, const std::string& shot_scale);
  // Reconstructions and their scales (bundle_adjuster.cc:219-244): a
  // reconstruction holds one scale per instance, or one shared by all of
  // them; constant or optimised (the lower bound 0 of the reference is not
  // enforced).  Unknown reconstruction ids are ignored, as in the reference.
  void AddReconstruction(const std::string& id, bool constant);
  void AddReconstructionInstance(const std::string& reconstruction_id, double scale, const std::string& instance_id);
  void SetScaleSharing(const std::string& id, bool share);
  // Reconstruction::GetScale: the shared scale, or the instance's
  double GetReconstructionScale(const std::string& reconstruction_id, const std::string& instance_id) const;
  bool HasReconstruction(const std::string& id) const { return reconstructions_.count(id) != 0; }
  // AddRelativeMotion (bundle_adjuster.cc:303-305, added at :872-910):
  // motion = [rx ry rz tx ty tz scale], scale_matrix 7 x 7 row-major (null:
  // identity)
  void AddRelativeMotion(const std::string& instance_i, const std::string& instance_j, const double* motion,
                         double robust_multiplier, bool observed_scale, const double* scale_matrix);
  // SetAdjustAbsolutePositionStd (bundle_adjuster.cc:402-404): the GPS
  // priors of each scale group are divided by a std multiplier that the run
  // optimises, regularised by StdDeviationConstraint (:772-838)
  void SetAdjustAbsolutePositionStd(bool adjust) { adjust_position_std_ = adjust; }
  // AddHeatmap / AddAbsolutePositionHeatmap (bundle_adjuster.cc:331-350):
  // a cost grid (row-major, `width` columns, `resolution` metres per cell)
  // and a shot's position looked up in it, centred at (x_offset, y_offset).
  void AddHeatmap(const std::string& id, const double* data, int64_t n, int64_t width, double resolution);
  void AddAbsolutePositionHeatmap(const std::string& shot, const std::string& heatmap_id, double x_offset,
                                  double y_offset, double std_deviation);
  void AddPointProjectionObservation(const std::string& shot, const std::string& point, const double* obs,
                                     double std_dev, bool is_gcp);
  // The depth_prior argument of AddPointProjectionObservation
  // (bundle_adjuster.cc:274-301; added as a RelativeDepthError block at Run,
  // :572-604): attaches map::Depth {value, is_radial, std_deviation} to the
  // observation added `index`-th (0-based).  The value and std are stored as
  // floats, as map::Depth holds them; a non-finite value makes Run throw.
  void SetObservationDepthPrior(int64_t index, double value, double std_dev, bool is_radial);
  // index-based adders (the raw-pointer path of AddPointProjectionObservationRaw)
  int64_t ShotIndex(const std::string& shot) const;
  int64_t PointIndex(const std::string& point) const;
  int64_t AddPointsBulk(int64_t n, const double* xyz, const uint8_t* constant, const char* const* ids);
  void AddObservationsBulk(int64_t n, const int32_t* shot, const int32_t* point, const double* xy,
                           const double* std_dev, const uint8_t* is_gcp);
  void SetCameraBias(const std::string& camera, const double* rotation, const double* translation, double scale);
  // SetCameraBias's parameters_to_optimize (bundle_adjuster.cc:131-140):
  // indices of Similarity::Parameter (RX RY RZ TX TY TZ SCALE, bias.h:12);
  // the GPS priors of the instances referencing the camera then take the
  // bias as unknowns (DataPriorError with SimilarityPriorTransform,
  // :806-838)
  void SetCameraBiasParameters(const std::string& camera, const int* indices, int n);
  // GetBias (bundle_adjuster.cc:1317-1323): rotation[3], translation[3], scale
  void GetBias(const std::string& camera, double* rotation, double* translation, double* scale) const;

  // settings (bundle_adjuster.cc:400-483, pybundle.pyi:131)
  void SetPointProjectionLossFunction(const std::string& name, double threshold);
  void SetIrlsMode(int mode) { opts_.irls = mode; }
  void SetPrecision(int p) { opts_.precision = p; }
  void SetMaxNumIterations(int n) { opts_.max_iterations = n; }
  void SetNumThreads(int n) { num_threads_ = n; }
  void SetUseAnalyticDerivatives(bool v) { use_analytic_ = v; }
  void SetLinearSolverType(const std::string& t) { opts_.linear_solver = t; }
  void SetInternalParametersPriorSD(double focal, double aspect, double c, double k1, double k2, double p1,
                                    double p2, double k3, double k4);
  void SetRigParametersPriorSD(double translation, double rotation);
  void SetComputeReprojectionErrors(bool v) { opts_.compute_reprojection_errors = v; }
  void SetComputeCovariances(bool v) { compute_covariances_ = v; }
  void SetSkipInitialReweighting(bool v) { opts_.skip_initial_reweighting = v; }
  void SetDefaultDensityRatio(double r) { opts_.default_density_ratio = r; }
  double GetDefaultDensityRatio() const { return opts_.default_density_ratio; }
  void SetGroupDensityRatio(const std::string& g, double r) { group_ratio_[g] = r; }
  double GetGroupDensityRatio(const std::string& g) const;
  void SetPcgTolerance(double t) { opts_.pcg_tolerance = t; }
  void SetMatrixFree(int mode) { opts_.matrix_free = mode; }
  void SetPcgGraph(bool enable) { opts_.pcg_graph = enable; }
  void SetCoarsePreconditioner(int leaf) { opts_.coarse_leaf = leaf; }
  // the coarse space a run would build (the run-time set-up, no solve)
  CoarseSpace CoarseLayout(int leaf);
  // Point-partitioned solve over `world` ranks (one per GPU): every rank
  // holds the whole problem, and this one solves with the points of
  // ShardRange(rank) and all of their observations, exchanging the
  // camera-side sums through `allreduce` (ShardComm, problem.h).  After the
  // run every rank holds the same cameras, rig cameras and instances, and
  // the solved values of its own points; the other points keep their values
  // from before the run.
  void SetShard(int rank, int world, int (*allreduce)(void*, double*, int64_t, int), void* ctx);
  // Points [first, last) of a rank: contiguous ranges of point indices with
  // nearly equal numbers of observations (a function of the problem only, so
  // every rank computes the same partition).
  std::pair<int64_t, int64_t> ShardRange(int rank) const;
  const ShardComm& Shard() const { return opts_.shard; }

  void Run();

  // Batched runs (gbba_batch_*): the run-time set-up of Run() without the
  // solve, the problem and options the batch solves, and the result of the
  // batch for this problem.
  void PrepareRun();
  // the rig cameras without the scale blocks a run set-up added
  void DropScaleBlocks();
  Problem& MutableProblem() { return problem_; }
  const SolverOptions& Options() const { return opts_; }
  void SetBatchResult(const SolveSummary& s, std::vector<double> errors);

  // getters (bundle_adjuster.cc:1303-1399)
  int GetCamera(const std::string& id, int* model, double* values, int cap) const;
  void GetRigInstancePose(const std::string& id, double* pose) const;
  void GetRigCameraPose(const std::string& id, double* pose) const;
  void GetPoint(const std::string& id, double* p) const;
  bool HasPoint(const std::string& id) const { return point_index_.count(id) != 0; }
  int64_t NumProjections() const { return int64_t(problem_.observations.size()); }
  int64_t NumPoints() const { return int64_t(problem_.points.size()); }
  void GetPointsBulk(int64_t first, int64_t n, double* xyz) const;
  void GetProjectionResults(int64_t n, double* errors, double* weights, int32_t* dims) const;
  // observation point indices in insertion order (for the outlier selection)
  std::vector<int32_t> ObservationPoints() const;
  int64_t NumObservations() const { return int64_t(problem_.observations.size()); }
  bool HasResults() const { return has_run_ && errors_.size() == 3 * problem_.observations.size(); }
  const std::vector<double>& Errors() const { return errors_; }
  const std::vector<double>& Weights() const { return weights_; }
  bool CovarianceValid() const { return covariance_valid_; }
  // The 6 x 6 covariance (row-major) of a rig instance's pose
  // [rx ry rz tx ty tz] from the last run with covariances on: the computed
  // block, or the reference's default (1e-5 rotation, 1e-2 translation
  // variances) when the estimation failed.
  void GetRigInstanceCovariance(const std::string& id, double* out) const;
  std::string BriefReport() const;
  std::string FullReport() const;
  std::string IrlsReport() const;
  const SolveSummary& Summary() const { return summary_; }

 private:
  void camera_sigma(CameraBlock& c) const;

  Problem problem_;
  SolverOptions opts_;
  std::unordered_map<std::string, int> camera_index_, rig_camera_index_, instance_index_, shot_index_;
  std::unordered_map<std::string, int64_t> point_index_;
  std::vector<std::string> shot_ids_;
  std::map<std::string, double> group_ratio_;
  std::vector<std::string> scale_groups_;
  double focal_sd_ = 1, aspect_sd_ = 1, c_sd_ = 1, k1_sd_ = 1, k2_sd_ = 1, p1_sd_ = 1, p2_sd_ = 1, k3_sd_ = 1,
         k4_sd_ = 1;
  double rig_translation_sd_ = 1.0, rig_rotation_sd_ = 1.0;
  int num_threads_ = 1;
  bool use_analytic_ = false;
  bool compute_covariances_ = false;
  bool covariance_valid_ = false;
  std::vector<double> covariances_;  // [n_instances][36], empty until a run computes them
  struct PendingOrientation {
    std::string shot;
    int kind;
    double value[3];
    double std_deviation;
  };
  std::vector<PendingOrientation> orientations_;
  struct PendingRelative {
    int kind;
    std::string shots[3];
    double rotation[3];
    double scale_matrix[9];
    double margin, std_deviation, alpha, position_std, orientation_std;
  };
  std::vector<PendingRelative> relatives_;
  std::string relative_loss_name_ = "CauchyLoss";
  struct ReconstructionScales {
    std::map<std::string, double> scales;  // instance id -> scale (std::map: the first is the shared one)
    bool constant = false;
    bool shared = true;
  };
  std::map<std::string, ReconstructionScales> reconstructions_;
  std::unordered_map<std::string, std::string> reconstruction_of_;  // instance id -> reconstruction id
  struct PendingMotion {
    std::string instances[2];
    double motion[7];
    double scale_matrix[49];
    double robust_multiplier;
    bool observed_scale;
  };
  std::vector<PendingMotion> motions_;
  // the scale blocks of the last run: (reconstruction, instance key, rig-camera block)
  struct ScaleBlock {
    std::string reconstruction, instance;  // empty for a GPS std multiplier
    int block;
    bool reconstruction_scale = true;
    int bias_camera = -1;  // >= 0: the camera's optimised bias (pose block; scale block = block + 1)
  };
  std::vector<ScaleBlock> scale_blocks_;
  bool adjust_position_std_ = false;
  std::vector<int> moved_priors_;  // instances whose GPS prior a run turned into a host term
  size_t n_rig_cameras_ = 0;  // rig cameras before the scale blocks
  std::unordered_map<std::string, int> heatmap_index_;
  struct PendingHeatmap {
    std::string shot;
    int heatmap;
    double x_offset, y_offset, std_deviation;
  };
  std::vector<PendingHeatmap> heatmap_terms_;
  bool has_gauge_ = false;
  std::string gauge_shots_[2];
  double relative_loss_threshold_ = 1.0;
  std::string loss_name_ = "TrivialLoss";
  SolveSummary summary_;
  std::vector<double> errors_, weights_;
  bool has_run_ = false;
};

// Parameter types of a camera model in geometry::Camera order
// (camera.cc:11-172), as geometry::Camera::Parameters values.
enum CameraParam {
  kParamTransition, kParamK1, kParamK2, kParamK3, kParamK4, kParamK5, kParamK6, kParamP1, kParamP2,
  kParamFocal, kParamAspectRatio, kParamCx, kParamCy, kParamS0, kParamS1, kParamS2, kParamS3, kParamNone
};
std::vector<int> camera_parameter_types(int model);

}  // namespace gbba
