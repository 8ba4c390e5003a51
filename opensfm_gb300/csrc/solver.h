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
};

// precision 0: FP64; otherwise mixed FP32/FP64.
std::unique_ptr<SolverBase> make_solver(int precision);
std::unique_ptr<SolverBase> make_solver_fp64();
std::unique_ptr<SolverBase> make_solver_mixed();

}  // namespace gbba
