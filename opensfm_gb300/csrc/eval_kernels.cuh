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

// Observation record: observed coordinates, 1/std and the shot index
// (16 B in FP32, 32 B in FP64), read with vector loads.  A depth prior of
// the solver (RelativeDepthError) rides on a slot of its own with
// x = the prior depth, y = 1 when the depth is radial (0: the camera-frame
// z) and w = -1/std: a negative weight marks it.
template <typename R>
struct ObsPack;

// What a solver slot holds: a projection, a ground-control projection
// (IRLS group GCP2D) or a depth prior (group DEPTH).
enum SlotKind : uint8_t { kSlotProjection = 0, kSlotGcp = 1, kSlotDepth = 2 };
template <>
struct alignas(16) ObsPack<float> {
  float x, y, w;
  int32_t shot;
};
template <>
struct alignas(16) ObsPack<double> {
  double x, y, w;
  int32_t shot, pad;
};

// Cameras up to this count are staged in shared memory by the kernels.
constexpr int kSharedCameras = 64;

// Device view of the geometry needed to evaluate observations.  Observation
// arrays are indexed by slot (the solver's point-major padded order; the
// standalone evaluator uses the caller's order).  obs_point < 0 marks a
// padding slot.
template <typename R>
struct SceneView {
  int64_t n_slots;
  int n_cameras;
  const ShotGeom<R>* geom;                      // [n_shots]
  const RigGeom<R>* rig;                        // [n_shots] or null
  const int* cam_model;                         // [n_cameras]
  const R* cam_params;                          // [n_cameras][16]
  const typename PointStore<R>::type* points;   // [n_points]
  const ObsPack<R>* obs;                        // [n_slots]
  const int* obs_point;                         // [n_slots]
};

// Stages the camera parameters (and models) in shared memory when they fit.
template <typename R>
__device__ __forceinline__ const R* stage_cameras(const SceneView<R>& s, R* smem_params, int* smem_models,
                                                  const int*& models) {
  if (s.n_cameras <= kSharedCameras) {
    for (int i = threadIdx.x; i < s.n_cameras * kMaxCameraParams; i += blockDim.x) smem_params[i] = s.cam_params[i];
    for (int i = threadIdx.x; i < s.n_cameras; i += blockDim.x) smem_models[i] = s.cam_model[i];
    __syncthreads();
    models = smem_models;
    return smem_params;
  }
  models = s.cam_model;
  return s.cam_params;
}

// Second-level gathers of one observation (shot geometry, world point)
// once its observation record and point index are known.
template <typename R, int M>
__device__ __forceinline__ void load_inputs(const SceneView<R>& s, const ObsPack<R>& ob, int pt, const R* cams,
                                            const int* models, ObsInputs<R>& in) {
  in.ox = ob.x;
  in.oy = ob.y;
  in.w = ob.w;
  const int sh = ob.shot;
  ldg_copy(s.geom + sh, in.g);
  centred(s.points + pt, in.g, in.v);
  in.rg = s.rig ? s.rig + sh : nullptr;
  const int cam = int(in.g.cam);
  in.model = M >= 0 ? M : models[cam];
  in.cam = cams + cam * kMaxCameraParams;
}

// Per-shot precompute (FP64 in, working precision out).
template <typename R>
__global__ void shot_prep_kernel(int n_shots, const int* __restrict__ shot_inst,
                                 const int* __restrict__ shot_rig,
                                 const int* __restrict__ shot_cam,
                                 const double* __restrict__ inst_pose,
                                 const double* __restrict__ rig_pose,
                                 const uint8_t* __restrict__ rig_used, ShotGeom<R>* geom,
                                 RigGeom<R>* rig) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n_shots) return;
  const double* pi = inst_pose + 6 * shot_inst[s];
  double Ri[9], Ji[9];
  pose_rotation(pi, Ri, Ji);
  const int rc = shot_rig[s];
  const bool use_rig = rc >= 0 && rig_used[rc];
  double rot[9], tc[3] = {0.0, 0.0, 0.0};
  double Rr[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1}, Jr[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1}, cr[3] = {0.0, 0.0, 0.0};
  if (use_rig) {
    const double* pr = rig_pose + 6 * rc;
    pose_rotation(pr, Rr, Jr);
    cr[0] = pr[3]; cr[1] = pr[4]; cr[2] = pr[5];
    for (int m = 0; m < 3; ++m) {
      for (int j = 0; j < 3; ++j) {
        double a = 0.0;
        for (int n = 0; n < 3; ++n) a += Rr[m * 3 + n] * Ri[n * 3 + j];
        rot[m * 3 + j] = a;
      }
      tc[m] = -(Rr[m * 3 + 0] * cr[0] + Rr[m * 3 + 1] * cr[1] + Rr[m * 3 + 2] * cr[2]);
    }
  } else {
    for (int i = 0; i < 9; ++i) rot[i] = Ri[i];
  }
  ShotGeom<R> g;
  for (int i = 0; i < 9; ++i) {
    g.rot[i] = R(rot[i]);
    g.jr[i] = R(Ji[i]);
  }
  for (int i = 0; i < 3; ++i) g.tc[i] = R(tc[i]);
  g.cam = R(shot_cam[s]);
  g.inst = R(shot_inst[s]);
  g.rig = R(use_rig ? rc : -1);
  for (int i = 0; i < 3; ++i) {
    g.chi[i] = R(pi[3 + i]);
    g.clo[i] = R(pi[3 + i] - double(g.chi[i]));
  }
  for (int i = 0; i < int(sizeof(g.pad) / sizeof(R)); ++i) g.pad[i] = R(0);
  geom[s] = g;
  if (rig) {
    RigGeom<R> q;
    for (int i = 0; i < 9; ++i) {
      q.rinst[i] = R(Ri[i]);
      q.rrc[i] = R(Rr[i]);
      q.jrc[i] = R(Jr[i]);
    }
    for (int i = 0; i < 3; ++i) q.crc[i] = R(cr[i]);
    q.pad[0] = q.pad[1] = R(0);
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
  __shared__ R s_cam[kSharedCameras * kMaxCameraParams];
  __shared__ int s_model[kSharedCameras];
  const int* models;
  const R* cams = stage_cameras(s, s_cam, s_model, models);
  const int64_t stride = int64_t(gridDim.x) * blockDim.x;
  int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  // The observation record and point index of the next slot are loaded
  // one iteration ahead, so only the dependent gathers (shot geometry,
  // world point) sit on the critical path of an iteration.
  ObsPack<R> ob_next;
  int pt_next = -1;
  if (i < s.n_slots) {
    ldg_copy(s.obs + i, ob_next);
    pt_next = __ldg(s.obs_point + i);
  }
  for (; i < s.n_slots; i += stride) {
    const ObsPack<R> ob = ob_next;
    const int pt = pt_next;
    if (i + stride < s.n_slots) {
      ldg_copy(s.obs + i + stride, ob_next);
      pt_next = __ldg(s.obs_point + i + stride);
    }
    R rec[NP * VN];
    if (pt >= 0) {
      ObsInputs<R> in;
      load_inputs<R, M>(s, ob, pt, cams, models, in);
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
