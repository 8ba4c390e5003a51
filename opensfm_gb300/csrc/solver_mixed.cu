// The GPU solver instantiated in mixed precision (FP32 records, products
// and PCG vectors; FP64 centring, residuals, cost, gradient sums and state).
#include "solver_impl.cuh"

namespace gbba {

std::unique_ptr<SolverBase> make_solver_mixed() { return std::unique_ptr<SolverBase>(new DeviceSolver<float>()); }

std::unique_ptr<SolverBase> make_solver(int precision) {
  return precision == 0 ? make_solver_fp64() : make_solver_mixed();
}

}  // namespace gbba

namespace gbba {

std::unique_ptr<BatchSolverBase> make_batch_solver_mixed() {
  return std::unique_ptr<BatchSolverBase>(new BatchSolver<float>());
}

std::unique_ptr<BatchSolverBase> make_batch_solver(int precision) {
  return precision == 0 ? make_batch_solver_fp64() : make_batch_solver_mixed();
}

}  // namespace gbba
