// The GPU solver instantiated in FP64 (every record, product and vector in
// double precision).
#include "solver_impl.cuh"

namespace gbba {

std::unique_ptr<SolverBase> make_solver_fp64() { return std::unique_ptr<SolverBase>(new DeviceSolver<double>()); }

}  // namespace gbba

namespace gbba {

std::unique_ptr<BatchSolverBase> make_batch_solver_fp64() {
  return std::unique_ptr<BatchSolverBase>(new BatchSolver<double>());
}

}  // namespace gbba
