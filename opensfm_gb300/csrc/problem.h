// Host-side description of a bundle-adjustment problem in flat arrays.
//
// Built by the BundleAdjuster (string-id API, bundle_adjuster.cc:107-301)
// and consumed by the device solver.  Parameter blocks follow the
// reference's data layout:
//   camera       geometry::Camera values (camera.cc:11-172), prior, sigma
//   rig camera   bundle::Pose [rx ry rz tx ty tz] camera-to-world (pose.h)
//   rig instance bundle::Pose, optional position prior (GPS) + scale group
//   point        [x y z], optional prior (GCP3D)
// Locking follows ApplyParameterLocking (bundle_adjuster.cc:30-52): a block
// whose parameters_to_optimize list is empty is constant; a full list is
// free; a partial list fixes the complement (SubsetManifold).  The masks
// below hold one flag per parameter (1 = optimised).
#pragma once

#include "host_terms.h"

#include <cstdint>
#include <string>
#include <vector>

namespace gbba {

enum LossKind { kLossTrivial = 0, kLossHuber = 1, kLossSoftLOne = 2, kLossCauchy = 3, kLossArctan = 4 };
enum IrlsMode { kIrlsNone = 0, kIrlsMixture = 1 };

struct CameraBlock {
  int model = 0;
  int n = 0;                  // parameter count
  double value[16] = {0};
  double prior[16] = {0};
  double sigma[16] = {0};     // prior standard deviations
  uint8_t free_mask[16] = {0};
  uint8_t log_prior[16] = {0};  // focal / aspect ratio priors are logarithmic
};

struct PoseBlock {
  double value[6] = {0};
  uint8_t free_mask[6] = {0};
  bool has_prior = false;     // rig cameras: full pose prior (RCAM)
  double prior[6] = {0};
  double sigma[6] = {0};
  // rig instances: position prior (GPS) on [tx ty tz]
  bool has_position_prior = false;
  double position_prior[3] = {0};
  double position_sigma[3] = {0};
  int scale_group = -1;
  int bias_camera = -1;       // camera whose bias transforms the GPS prior
  bool used = true;           // rig cameras: false when identity and fixed
  // a reconstruction scale (value[0]) held in a rig-camera block that no
  // shot references: camera-side unknowns for the relative motions
  bool scale_block = false;
};

struct PointBlock {
  double value[3] = {0};
  bool free = true;
  bool has_prior = false;
  double prior[3] = {0};
  double sigma[3] = {0};
  bool has_altitude = true;
};

struct Bias {
  // geometry::Similarity: rotation (angle-axis), translation, scale; the
  // bias maps the GPS prior p to s * R p + t (bias.h:34-54).
  double r[3] = {0, 0, 0};
  double t[3] = {0, 0, 0};
  double s = 1.0;
  // the parameters the run optimises (SetCameraBias's
  // parameters_to_optimize, Similarity::Parameter order RX RY RZ TX TY TZ
  // SCALE); none by default (AddCamera, bundle_adjuster.cc:121-128)
  uint8_t free_mask[7] = {0, 0, 0, 0, 0, 0, 0};
  bool optimised() const {
    for (uint8_t f : free_mask)
      if (f) return true;
    return false;
  }
};

struct Shot {
  int instance = -1;
  int rig_camera = -1;
  int camera = -1;
};

struct Observation {
  int shot = -1;
  int point = -1;
  double x = 0, y = 0;
  double std_dev = 1.0;
  bool is_gcp = false;
  // optional depth prior of the observation (map::Depth: value, is_radial,
  // std_deviation, stored as floats; map/observation.h:10-18): a second
  // residual, std^-1 (depth of the point in the camera - value), the depth
  // being the camera-frame z or, when radial, the distance to the camera
  // (RelativeDepthError, bundle/error/relative_depth_error.h)
  bool has_depth = false;
  bool depth_radial = true;
  float depth = 0.0f;
  float depth_std = 1.0f;
};

// Point-partitioned solve over several ranks (one process or thread per
// GPU).  Every rank holds all cameras, rig cameras and instances and a share
// of the points with all of their observations; the camera-side sums of the
// observations (gradient, Schur right-hand side, preconditioner blocks, the
// Schur product of every PCG iteration) and the scalar sums (cost, model
// decrease, IRLS statistics) are combined by `allreduce`.  The callback
// reduces `count` doubles in place across the ranks (op 0: sum, 1: max) and
// returns 0, or nonzero on failure; every rank calls it the same number of
// times with the same counts.
struct ShardComm {
  int rank = 0;
  int world = 1;
  int (*allreduce)(void* ctx, double* data, int64_t count, int op) = nullptr;
  void* ctx = nullptr;
  bool active() const { return world > 1 && allreduce != nullptr; }
};

struct SolverOptions {
  int max_iterations = 500;
  int loss = kLossTrivial;
  double loss_threshold = 1.0;
  int irls = kIrlsMixture;
  double default_density_ratio = 1e-3;
  bool skip_initial_reweighting = false;
  int precision = 1;          // 0 FP64, 1 mixed
  std::string linear_solver = "SPARSE_SCHUR";
  int dense_max_unknowns = 4096;  // dense reduced-camera Cholesky below this
  // Jacobian records: 0 stored when they fit in device memory (else
  // matrix-free), 1 always matrix-free, -1 always stored
  int matrix_free = 0;
  // pose covariances of the final state (the 6 x 6 instance blocks of the
  // inverse Gauss-Newton matrix); computed when the reduced camera system is
  // dense-sized (dense_max_unknowns)
  bool compute_covariances = false;
  double pcg_tolerance = 1e-3;    // relative residual of the reduced system
  bool pcg_graph = true;          // PCG iterations as one graph launch (false: kernel by kernel)
  // two-level PCG preconditioner: > 0 adds a coarse space of similarity
  // modes over spatial clusters of at most this many rig instances
  // (coarse_space.h); 0: block-Jacobi only
  int coarse_leaf = 0;
  int pcg_max_iterations = 500;
  bool compute_reprojection_errors = true;
  bool record_trace = true;
  ShardComm shard;  // world > 1: this rank's share of a point-partitioned solve
};

struct Problem {
  std::vector<CameraBlock> cameras;
  std::vector<Bias> biases;        // one per camera
  std::vector<PoseBlock> rig_cameras;
  std::vector<PoseBlock> instances;
  std::vector<Shot> shots;
  std::vector<PointBlock> points;
  std::vector<Observation> observations;
  // absolute orientation constraints (up vector, pan, tilt, roll)
  std::vector<OrientationTerm> orientation_terms;
  std::vector<RelativeTerm> relative_terms;
  int relative_loss = 3;  // loss of the relative rotations (kinds as the projection loss), scale below
  double relative_loss_threshold = 1.0;
  // IRLS density ratios: one per projection group (shot groups "PROJ_<shot>"
  // then "GCP2D"), and the prior groups.
  std::vector<double> group_density_ratio;
  double ratio_cam = 1e-3, ratio_rig = 1e-3, ratio_gps = 1e-3, ratio_gcp3d = 1e-3, ratio_depth = 1e-3;
  // UP PAN TILT ROLL ROT POS MOTION GAUGE HEATMAP REL GPS STDDEV
  double ratio_host[12] = {1e-3, 1e-3, 1e-3, 1e-3, 1e-3, 1e-3, 1e-3, 1e-3, 1e-3, 1e-3, 1e-3, 1e-3};
  // AddHeatmap grids (the relative terms of kind kHeatmap point into them)
  struct Heatmap {
    std::vector<double> data;
    int width = 0;
    double resolution = 1.0;
  };
  std::vector<Heatmap> heatmaps;
};

// One LM iteration as reported by the solver.
struct IterationRecord {
  int iteration = 0;
  double cost = 0;          // cost after the iteration
  double cost_change = 0;
  double gradient_max_norm = 0;
  double step_norm = 0;
  double radius = 0;
  double relative_decrease = 0;
  int linear_iterations = 0;
  bool success = false;
  double seconds = 0;       // wall time since the start of the solve
};

struct SolveSummary {
  double initial_cost = 0;
  double final_cost = 0;
  int iterations = 0;
  int successful_steps = 0;
  int unsuccessful_steps = 0;
  std::string termination = "NO_CONVERGENCE";
  bool usable = true;
  double seconds = 0;
  double linear_solver_seconds = 0;
  double jacobian_seconds = 0;
  double residual_seconds = 0;
  double setup_seconds = 0;  // slot sorts, uploads, device buffers
  int64_t kernel_launches = 0;
  int64_t pcg_refinements = 0;  // FP64 residual evaluations (mixed-precision iterative refinement)
  int64_t linear_solver_failures = 0;  // dense factorizations that found the damped system not positive definite
  bool matrix_free = false;      // the record passes evaluated the Jacobians instead of reading them
  // two-level preconditioner: clusters, colours of the probe set, and the
  // Schur products spent on probing the coarse matrix
  int coarse_clusters = 0, coarse_colours = 0;
  int64_t coarse_probes = 0;
  std::string linear_solver;
  std::vector<IterationRecord> trace;
  std::vector<std::string> irls_lines;
};

}  // namespace gbba
