// Launches of the solver's record passes for a kernel configuration and a
// record source (stored planes, or matrix-free evaluation).  The stored
// launches are instantiated with the solver; the matrix-free ones in their
// own translation units (solver_mf_fp64.cu, solver_mf_mixed.cu) through
// launch_evaluated().
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "kernel_config.cuh"
#include "record_source.cuh"
#include "solver_kernels.cuh"
#include "solver_shot_major.cuh"

namespace gbba {

template <typename R>
struct RecordPassArgs {
  enum Which { kSchurRhs, kPointPass, kCameraPass, kModelChange, kPointPass64, kCameraPass64, kPermute };
  Which which;
  SolveView<R> v;
  ShotMajorView<R> sm{};
  int grid = 1;
  const R* x = nullptr;
  R* out = nullptr;
  const R* zbuf = nullptr;
  const R* dp = nullptr;
  double* dout = nullptr;
  const double* x64 = nullptr;
  const double* zbuf64 = nullptr;
  PrecondView<R> pc{};
  uint64_t plane_mask = 0;  // kPermute: shot-major planes to write
  cudaStream_t stream = 0;  // the stream the pass is launched on

  template <int M, int NR, int CMAX, bool RIG, typename Src>
  void launch(const Src& recs) const {
    const int g = grid;
    const cudaStream_t s = stream;
    switch (which) {
      case kSchurRhs:
        schur_rhs_precond_sm_kernel<R, NR, CMAX, RIG, Src><<<g, 256, 0, s>>>(v, sm, recs, dout, pc);
        break;
      case kPointPass: schur_point_pass_kernel<R, R, NR, CMAX, RIG, Src><<<g, 256, 0, s>>>(v, recs, x, out); break;
      case kCameraPass:
        schur_camera_pass_sm_kernel<R, R, NR, CMAX, RIG, Src><<<g, 256, 0, s>>>(v, sm, recs, x, zbuf, out);
        break;
      case kPointPass64:
        schur_point_pass_kernel<R, double, NR, CMAX, RIG, Src><<<g, 256, 0, s>>>(v, recs, x64, dout);
        break;
      case kCameraPass64:
        schur_camera_pass_sm_kernel<R, double, NR, CMAX, RIG, Src><<<g, 256, 0, s>>>(v, sm, recs, x64, zbuf64, dout);
        break;
      case kModelChange: model_change_kernel<R, NR, CMAX, RIG, Src><<<g, 256, 0, s>>>(v, recs, x, dp, dout); break;
      case kPermute:
        permute_records_kernel<R, NR, CMAX, RIG, Src><<<g, 256, 0, s>>>(v, sm, recs, plane_mask);
        break;
    }
  }
};

// The pass with records evaluated in place (matrix-free).
template <typename R>
void launch_evaluated(const KernelConfig& kc, const RecordPassArgs<R>& a);
template <>
void launch_evaluated<float>(const KernelConfig& kc, const RecordPassArgs<float>& a);
template <>
void launch_evaluated<double>(const KernelConfig& kc, const RecordPassArgs<double>& a);

}  // namespace gbba
