// Kernels shared by the standalone evaluator and the LM solver:
// shot precompute and the per-observation residual/Jacobian record writer.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "geometry_device.cuh"

namespace gbba {

// 16-byte vector type of a working precision: one "plane" of a record.
template <typename R> struct Vec16;
template <> struct Vec16<float> {
  using type = float4;
  static constexpr int kN = 4;
};
template <> struct Vec16<double> {
  using type = double2;
  static constexpr int kN = 2;
};

template <typename R>
__device__ __forceinline__ void store_plane(typename Vec16<R>::type* dst, const R* src);
template <>
__device__ __forceinline__ void store_plane<float>(float4* dst, const float* s) {
  *dst = make_float4(s[0], s[1], s[2], s[3]);
}
template <>
__device__ __forceinline__ void store_plane<double>(double2* dst, const double* s) {
  *dst = make_double2(s[0], s[1]);
}
template <typename R>
__device__ __forceinline__ void load_plane(const typename Vec16<R>::type* src, R* d);
template <>
__device__ __forceinline__ void load_plane<float>(const float4* s, float* d) {
  const float4 v = __ldg(s);
  d[0] = v.x; d[1] = v.y; d[2] = v.z; d[3] = v.w;
}
template <>
__device__ __forceinline__ void load_plane<double>(const double2* s, double* d) {
  const double2 v = __ldg(s);
  d[0] = v.x; d[1] = v.y;
}

// Number of 16-byte planes of a record of `width` scalars of type R.
template <typename R>
constexpr int planes_of(int width) {
  return (width + Vec16<R>::kN - 1) / Vec16<R>::kN;
}

// Device view of the geometry needed to evaluate observations.  Observation
// arrays are indexed by slot (the solver's point-major padded order; the
// standalone evaluator uses the caller's order).  obs_point < 0 marks a
// padding slot.
template <typename R>
struct SceneView {
  int64_t n_slots;
  const ShotGeom<R>* geom;     // [n_shots]
  const RigGeom<R>* rig;       // [n_shots] or null
  const Point4* center;       // [n_shots] rig instance centre (FP64)
  const int* shot_cam;         // [n_shots]
  const int* cam_model;        // [n_cameras]
  const R* cam_params;         // [n_cameras][16]
  const Point4* points;       // [n_points]
  const int* obs_shot;         // [n_slots]
  const int* obs_point;        // [n_slots]
  const R* obs_xy;             // [n_slots][2]
  const R* obs_w;              // [n_slots] 1 / std
};

template <typename R>
__device__ __forceinline__ ObsInputs<R> load_inputs(const SceneView<R>& s, int64_t i, int pt) {
  ObsInputs<R> in;
  const int sh = __ldg(s.obs_shot + i);
  in.ox = s.obs_xy[2 * i];
  in.oy = s.obs_xy[2 * i + 1];
  in.w = s.obs_w[i];
  const Point4 X = ldg_point4(s.points + pt);
  in.X[0] = X.x; in.X[1] = X.y; in.X[2] = X.z;
  const Point4 c = ldg_point4(s.center + sh);
  in.c[0] = c.x; in.c[1] = c.y; in.c[2] = c.z;
  in.g = s.geom + sh;
  in.rg = s.rig ? s.rig + sh : nullptr;
  const int cam = __ldg(s.shot_cam + sh);
  in.model = __ldg(s.cam_model + cam);
  in.cam = s.cam_params + cam * kMaxCameraParams;
  return in;
}

// Per-shot precompute (FP64 in, working precision out).
template <typename R>
__global__ void shot_prep_kernel(int n_shots, const int* __restrict__ shot_inst,
                                 const int* __restrict__ shot_rig,
                                 const double* __restrict__ inst_pose,
                                 const double* __restrict__ rig_pose,
                                 const uint8_t* __restrict__ rig_used, ShotGeom<R>* geom,
                                 Point4* center, RigGeom<R>* rig) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n_shots) return;
  const double* pi = inst_pose + 6 * shot_inst[s];
  double Ri[9], dRi[27];
  pose_rotation(pi, Ri, dRi);
  const int rc = shot_rig[s];
  const bool use_rig = rc >= 0 && rig_used[rc];
  double rot[9], drot[27], tc[3] = {0.0, 0.0, 0.0};
  double Rr[9], dRr[27], cr[3] = {0.0, 0.0, 0.0};
  if (use_rig) {
    const double* pr = rig_pose + 6 * rc;
    pose_rotation(pr, Rr, dRr);
    cr[0] = pr[3]; cr[1] = pr[4]; cr[2] = pr[5];
    for (int m = 0; m < 3; ++m) {
      for (int j = 0; j < 3; ++j) {
        double a = 0.0;
        for (int n = 0; n < 3; ++n) a += Rr[m * 3 + n] * Ri[n * 3 + j];
        rot[m * 3 + j] = a;
        for (int k = 0; k < 3; ++k) {
          double b = 0.0;
          for (int n = 0; n < 3; ++n) b += Rr[m * 3 + n] * dRi[(n * 3 + j) * 3 + k];
          drot[(m * 3 + j) * 3 + k] = b;
        }
      }
      tc[m] = -(Rr[m * 3 + 0] * cr[0] + Rr[m * 3 + 1] * cr[1] + Rr[m * 3 + 2] * cr[2]);
    }
  } else {
    for (int i = 0; i < 9; ++i) rot[i] = Ri[i];
    for (int i = 0; i < 27; ++i) drot[i] = dRi[i];
    for (int i = 0; i < 9; ++i) Rr[i] = (i % 4 == 0) ? 1.0 : 0.0;
    for (int i = 0; i < 27; ++i) dRr[i] = 0.0;
  }
  ShotGeom<R> g;
  for (int i = 0; i < 9; ++i) g.rot[i] = R(rot[i]);
  for (int i = 0; i < 27; ++i) g.drot[i] = R(drot[i]);
  for (int i = 0; i < 3; ++i) g.tc[i] = R(tc[i]);
  g.pad = R(0);
  geom[s] = g;
  center[s] = Point4{pi[3], pi[4], pi[5], 0.0};
  if (rig) {
    RigGeom<R> q;
    for (int i = 0; i < 9; ++i) {
      q.rinst[i] = R(Ri[i]);
      q.rrc[i] = R(Rr[i]);
    }
    for (int i = 0; i < 27; ++i) q.drrc[i] = R(dRr[i]);
    for (int i = 0; i < 3; ++i) q.crc[i] = R(cr[i]);
    rig[s] = q;
  }
}

// Writes the residual/Jacobian record of every slot as 16-byte planes:
// plane p of slot i lives at out[p * plane_stride + i], so each plane is a
// fully coalesced stream.  Planes whose bit is clear in plane_mask are not
// written (blocks of fixed parameters).
template <typename R, int M, int NR, int CMAX, bool RIG>
__global__ void __launch_bounds__(256) eval_records_kernel(SceneView<R> s,
                                                           typename Vec16<R>::type* __restrict__ out,
                                                           int64_t plane_stride, uint64_t plane_mask) {
  using L = RecordLayout<NR, CMAX, RIG>;
  constexpr int NP = planes_of<R>(L::kWidth);
  constexpr int VN = Vec16<R>::kN;
  const int64_t stride = int64_t(gridDim.x) * blockDim.x;
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < s.n_slots; i += stride) {
    R rec[NP * VN];
    const int pt = __ldg(s.obs_point + i);
    if (pt >= 0) {
      const ObsInputs<R> in = load_inputs(s, i, pt);
      eval_observation<R, M, NR, CMAX, RIG, true>(in, rec);
#pragma unroll
      for (int k = L::kWidth; k < NP * VN; ++k) rec[k] = R(0);
    } else {
#pragma unroll
      for (int k = 0; k < NP * VN; ++k) rec[k] = R(0);
    }
#pragma unroll
    for (int p = 0; p < NP; ++p) {
      if (plane_mask & (uint64_t(1) << p)) store_plane<R>(out + p * plane_stride + i, rec + p * VN);
    }
  }
}

}  // namespace gbba
