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
#include "record_stage.cuh"
#include "solver_kernels.cuh"
#include "solver_shot_major.cuh"

namespace gbba {

// Streaming multiprocessors of the current device (read once, before any
// stream capture: solver setup calls it).
inline int device_sm_count() {
  static const int n = [] {
    int dev = 0, v = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
      return 1;
    return v > 0 ? v : 1;
  }();
  return n;
}

// Raises the dynamic shared-memory limit of the staged Schur-product
// kernels of one configuration (once, at solver setup: outside any capture).
template <typename R>
struct StagedPrepare {
  template <int M, int NR, int CMAX, bool RIG>
  void run() {
    if constexpr (staged_record_fits<R, NR, CMAX, RIG>()) {
      constexpr int bytes = staged_smem_bytes<R, planes_of<R>(RecordLayout<NR, CMAX, RIG>::kWidth)>();
      cudaFuncSetAttribute(staged_point_pass_kernel<R, R, NR, CMAX, RIG>,
                           cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
      cudaFuncSetAttribute(staged_camera_pass_kernel<R, R, NR, CMAX, RIG>,
                           cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    }
    device_sm_count();
  }
};

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
    if constexpr (Src::kPrefetch && staged_record_fits<R, NR, CMAX, RIG>()) {
      // a single problem's stored records: the PCG's Schur-product passes
      // stage them through shared memory (record_stage.cuh), one grid of
      // resident blocks (the FP64 products of iterative refinement keep the
      // register pipeline)
      constexpr int bytes = staged_smem_bytes<R, planes_of<R>(RecordLayout<NR, CMAX, RIG>::kWidth)>();
      const int g1 = device_sm_count() * staged_min_blocks<R, R, NR, CMAX, RIG>();
      if (which == kPointPass) {
        staged_point_pass_kernel<R, R, NR, CMAX, RIG><<<g < g1 ? g : g1, kStagedBlock, bytes, s>>>(
            v, recs.pm, recs.stride, x, out);
        return;
      }
      if (which == kCameraPass) {
        staged_camera_pass_kernel<R, R, NR, CMAX, RIG><<<g < g1 ? g : g1, kStagedBlock, bytes, s>>>(
            v, sm, recs.stride, x, zbuf, out);
        return;
      }
    }
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
