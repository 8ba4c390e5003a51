// Where the solver's record passes get the residual + Jacobian record of an
// observation.
//
//   StoredRecords     the record planes written once per linearization:
//                     point-major by linearize_kernel, shot-major by
//                     permute_records_kernel (112 B per observation and copy
//                     for a perspective camera in FP32).
//   EvaluatedRecords  matrix-free: the observation is evaluated again in
//                     every pass -- the same evaluation, FP64 residual and
//                     robust correction as linearize_kernel -- so no record
//                     is stored.  The solver uses it when the two record
//                     copies would not fit in device memory, or on request.
//
// The passes take the source as a template parameter: point_major(i) is the
// record of point-major slot i; shot_major(j, src) that of shot-major slot j,
// whose point-major slot is src.
#pragma once

#include "solver_kernels.cuh"

namespace gbba {

template <typename R, int NP, bool PREFETCH = true>
struct StoredRecords {
  // every slot, padding included, has a record: the passes may load it
  // before they know whether the slot is valid (one iteration ahead).  The
  // batched solver turns this off: it reads only the records of problems
  // still running, and the extra registers of the pipeline cost it more
  // than they gain.
  static constexpr bool kPrefetch = PREFETCH;
  const typename Vec16<R>::type* pm;
  const typename Vec16<R>::type* sm;
  int64_t stride;
  __device__ __forceinline__ void point_major(const SolveView<R>&, int64_t i, R* rec) const {
    load_record<R, NP>(pm, stride, i, rec);
  }
  __device__ __forceinline__ void shot_major(const SolveView<R>&, int64_t j, int64_t, R* rec) const {
    load_record<R, NP>(sm, stride, j, rec);
  }
};

template <typename R, int M, int NR, int CMAX, bool RIG>
struct EvaluatedRecords {
  static constexpr bool kPrefetch = false;  // padding slots cannot be evaluated
  __device__ __forceinline__ void point_major(const SolveView<R>& v, int64_t i, R* rec) const { eval(v, i, rec); }
  __device__ __forceinline__ void shot_major(const SolveView<R>& v, int64_t, int64_t src, R* rec) const {
    eval(v, src, rec);
  }
  static __device__ __forceinline__ void eval(const SolveView<R>& v, int64_t i, R* rec) {
    using L = RecordLayout<NR, CMAX, RIG>;
    constexpr int NP = planes_of<R>(L::kWidth);
    constexpr int VN = Vec16<R>::kN;
#pragma unroll
    for (int k = 0; k < NP * VN; ++k) rec[k] = R(0);
    const SceneView<R>& s = v.scene;
    ObsPack<R> ob;
    ldg_copy(s.obs + i, ob);
    ObsInputs<R> in;
    load_inputs<R, M>(s, ob, s.obs_point[i], s.cam_params, s.cam_model, in);
    eval_observation<R, M, NR, CMAX, RIG, true, true>(in, rec);
    if (v.resid64) {
#pragma unroll
      for (int q = 0; q < NR; ++q) rec[L::kR + q] = R(v.resid64[4 * i + q]);
    }
    robust_correct<R, NR, CMAX, RIG>(v.loss, v.loss_a, v.weight[i], rec);
  }
};

}  // namespace gbba
