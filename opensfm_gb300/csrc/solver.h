// Levenberg-Marquardt bundle-adjustment solver on the GPU.
//
// The trust-region loop follows the behaviour the reference configures for
// Ceres (bundle_adjuster.cc:1159-1190, irls_solver.cc:406-474), restated from
// Ceres Solver's public documentation:
//   * LEVENBERG_MARQUARDT strategy, initial radius 1e4, radius capped at 1e8
//     (IRLS run options), step accepted when the ratio of actual to model
//     cost decrease exceeds 1e-3; on success radius /= max(1/3, 1-(2 rho-1)^3)
//     and the decrease factor resets to 2, on failure radius /= factor and
//     the factor doubles;
//   * Jacobi column scaling computed at the first iteration, LM diagonal
//     clamped to [1e-6, 1e32];
//   * the IRLS schedule of IRLSIterationCallback (irls_solver.cc:93-188):
//     reweight every max_iterations/10 successful iterations or on inner
//     convergence (function 1e-7, gradient 1e-10, parameter 1e-8), stop when
//     the log-likelihood changes by less than 1e-3 relative.
// After a reweighting the cost and linearization are recomputed with the
// new weights (the objective changed).
#pragma once

#include <memory>

#include "problem.h"

namespace gbba {

class SolverBase {
 public:
  virtual ~SolverBase() = default;
  // Runs the optimisation; updates `problem` in place.
  virtual SolveSummary solve(Problem& problem, const SolverOptions& opts) = 0;
  // Per-observation unscaled residuals (std = 1) and IRLS weights of the
  // last solve, in the order of problem.observations.
  virtual void reprojection(std::vector<double>& errors /* n x 3 */, std::vector<double>& weights) = 0;
  // Pose covariances of the rig instances ([n_instances][6][6]) when the
  // options asked for them; false if they could not be computed.
  virtual bool covariances(std::vector<double>& cov) {
    cov.clear();
    return false;
  }
};

// Many independent problems solved together (batched local bundle
// adjustment): see batch_loop.inc.
struct BatchOptions {
  int max_iterations = 50;
  int loss = kLossTrivial;
  double loss_threshold = 1.0;
  int pcg_iterations = 50;           // per LM iteration (each problem stops at its tolerance)
  double pcg_tolerance = 1e-3;
  double function_tolerance = 1e-7;  // as the single-problem solver's inner convergence test
  // 2: the whole LM loop one CUDA graph launch (a device-side while node);
  // 1: one recorded LM iteration replayed per iteration; 0: plain launches
  int use_graph = 2;
  bool autotune = true;              // pick the slot-kernel grid by timing
};

struct BatchProblemSummary {
  double initial_cost = 0, final_cost = 0;
  int iterations = 0, successful_steps = 0, unsuccessful_steps = 0, pcg_iterations = 0;
  bool converged = false;
  std::vector<double> errors;  // n x 3 unscaled residuals of the final state
};

struct BatchSummary {
  std::vector<BatchProblemSummary> problems;
  double seconds = 0, setup_seconds = 0, solve_seconds = 0;
  int lm_iterations = 0;  // iterations of the batch (the slowest problem)
  int grid = 0;           // slot-kernel grid chosen by the autotuner
  int64_t graph_nodes = 0, kernel_launches = 0;
  int64_t graph_launches = 0;  // graph launches of the LM loop (1 with the device-side loop)
};

class BatchSolverBase {
 public:
  virtual ~BatchSolverBase() = default;
  // Optimises every problem; results are written back into the problems.
  virtual BatchSummary solve_batch(const std::vector<Problem*>& problems, const BatchOptions& opts) = 0;
};

std::unique_ptr<BatchSolverBase> make_batch_solver(int precision);
std::unique_ptr<BatchSolverBase> make_batch_solver_fp64();
std::unique_ptr<BatchSolverBase> make_batch_solver_mixed();

// Optimised camera-side coordinates of a problem: the free coordinates of
// the rig instances, of the rig cameras that some shot applies with a free
// coordinate (and of the scale blocks), and of the cameras.  The solver's
// explicit reduced camera system has this size.
inline int camera_side_unknowns(const Problem& P) {
  bool any_rig_free = false;
  for (const Shot& s : P.shots)
    if (s.rig_camera >= 0 && P.rig_cameras[s.rig_camera].used)
      for (int k = 0; k < 6; ++k) any_rig_free |= P.rig_cameras[s.rig_camera].free_mask[k] != 0;
  int n = 0;
  for (const PoseBlock& b : P.instances)
    for (int k = 0; k < 6; ++k) n += b.free_mask[k] != 0;
  for (const PoseBlock& b : P.rig_cameras)
    if (b.used && (any_rig_free || b.scale_block))
      for (int k = 0; k < 6; ++k) n += b.free_mask[k] != 0;
  for (const CameraBlock& c : P.cameras)
    for (int k = 0; k < c.n; ++k) n += c.free_mask[k] != 0;
  return n;
}

// Whether a solve takes exact steps from the explicit reduced camera system
// (dense mode): an exact linear solver type, a single rank, and at most
// opts.dense_max_unknowns camera-side unknowns.
inline bool exact_dense_steps(const Problem& P, const SolverOptions& opts) {
  const std::string& ls = opts.linear_solver;
  const bool exact = ls == "DENSE_SCHUR" || ls == "DENSE_QR" || ls == "DENSE_NORMAL_CHOLESKY" ||
                     ls == "SPARSE_SCHUR" || ls == "SPARSE_NORMAL_CHOLESKY";
  const int n = camera_side_unknowns(P);
  return exact && !opts.shard.active() && n > 0 && n <= opts.dense_max_unknowns;
}

// precision 0: FP64; otherwise mixed FP32/FP64.
std::unique_ptr<SolverBase> make_solver(int precision);
std::unique_ptr<SolverBase> make_solver_fp64();
std::unique_ptr<SolverBase> make_solver_mixed();

}  // namespace gbba
