// Dense symmetric positive definite solver for the reduced camera system.
//
// Ceres factors the reduced camera system S = U - W V^-1 W^T with a dense
// (DENSE_SCHUR) or sparse (SPARSE_SCHUR) Cholesky factorization
// (bundle_adjuster.cc:1159-1190; the choice in ba_helpers.cc:42-49).  Here
// S is Jacobi-scaled, converted to FP32 and factored by a blocked
// left-looking Cholesky whose block products run on the tensor cores
// (tcgen05, TF32 operands, three products per term); FP64 iterative
// refinement against the FP64 matrix then brings the solution to FP64
// accuracy.
#pragma once

#include <cuda_runtime.h>

#include "device_buffer.h"

namespace gbba {

struct DenseSolveStats {
  int status = 0;           // 0 solved, 1 not positive definite, 2 device wait timed out, 3 not converged
  int refinements = 0;      // FP64 conjugate-gradient iterations (one FP64 matrix product each)
  double rel_residual = 0;  // |D (b - A x)| / |D b| of the returned x, D = diag(A)^-1/2
};

class DenseSpdSolver {
 public:
  // Factors A: device FP64, n x n row-major with leading dimension lda.  The
  // lower triangle is read and the upper triangle is overwritten with its
  // mirror (the solve multiplies by the full matrix).  A must stay
  // unchanged until the last solve().  Returns a DenseSolveStats status
  // (0, 1 or 2).
  int factor(double* A, int n, int lda);
  // x = A^-1 b (device FP64 vectors of length n) to a relative scaled
  // residual tol within max_iterations FP64 conjugate-gradient iterations
  // preconditioned by the factor.
  int solve(const double* b, double* x, double tol, int max_iterations, DenseSolveStats* stats);
  // Columns of A^-1, up to kInverseBatch at a time by conjugate gradients
  // in lockstep (FP64, preconditioned by the factor, every column to the
  // relative scaled residual tol): column c solves A x = e_{unit[c]} and
  // returns x at the dense indices gather[6 c .. 6 c + 5] (-1: 0) in
  // out[6 c .. 6 c + 5].  Host arrays of m columns.  Returns 0, or 1 when a
  // column met p.Ap <= 0 or did not converge within max_iterations.
  // inv = D (L L^T)^-1 D, the inverse through the FP32 factor only (no
  // refinement), as an n x n FP32 row-major matrix with leading dimension
  // ld, symmetrized: the factor as a preconditioner, applied by one matrix
  // product.  The multi-right-hand-side triangular steps solve all columns
  // at once, 32 per CTA column of each step's grid.
  void explicit_inverse(float* inv, int ld);
  static constexpr int kInverseBatch = 32;
  int inverse_columns(const int* unit, int m, const int* gather, double* out, double tol, int max_iterations);
  int n() const { return n_; }
  double shift() const { return shift_; }  // diagonal shift the factor needed (0 normally)

 private:
  int n_ = 0, nt_ = 0, n_pad_ = 0, lda_ = 0;
  double shift_ = 0.0;
  double* A_ = nullptr;
  DeviceArray<float> L_, dinv_, rs_, ts_;
  DeviceArray<double> dscale_, r_, z_, scal_;
  DeviceArray<int> status_;
  // batched columns: FP64 x, r, p, q, z_new, z_old and FP32 rs, b, y, x, all
  // [n_pad][kInverseBatch] row-major, per-column scalars, index tables
  DeviceArray<double> mv_, mscal_, mout_;
  DeviceArray<float> mts_;
  DeviceArray<int> munit_, mgather_;
};

// C = A B^T on the tensor cores for row-major device FP32 matrices A (m x k,
// leading dimension lda), B (n x k, ldb), C (m x n, ldc); m and n multiples
// of 128, k a multiple of 32, leading dimensions multiples of 4.  status
// (device) is set to 2 if a device wait timed out.
void tc_gemm_nt(const float* A, int lda, const float* B, int ldb, float* C, int ldc, int m, int n, int k,
                int* status);

}  // namespace gbba
