// Projection + residual as a differentiable operation: the forward kernel
// (residuals, optionally the Jacobian records saved for the backward pass)
// and the adjoint kernel (J^T g accumulated into the gradients of the
// camera parameters, rig-instance poses and points), behind
// gbba_projection_forward / gbba_projection_backward.
//
// Per observation the forward is ReprojectionError2DAnalytic<C>::Evaluate
// (opensfm/src/lib/bundle/error/projection_errors.h:67-207) for a shot whose
// pose is its rig instance's (no rig camera); the adjoint contracts the
// same analytic Jacobian blocks with the incoming gradient.  In
// "recompute" mode the backward evaluates the Jacobian again instead of
// reading saved records (no per-observation memory kept between passes).
//
// Every array is device memory of the caller; the functions allocate
// nothing.  The scratch (per-shot geometry + status words) is sized by
// gbba_projection_scratch_bytes.
#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "../../include/gbba.h"
#include "capi_util.h"
#include "eval_kernels.cuh"
#include "solver_shot_major.cuh"

namespace gbba {
namespace {

constexpr int kAgDyn = -1;
constexpr size_t kAgStatusBytes = 256;

enum : unsigned long long {
  kAgBadShot = 1,      // shot references a missing instance or camera
  kAgBadModel = 2,     // unknown or spherical projection type
  kAgBadObs = 4,       // observation references a missing shot or point
  kAgBadStd = 8,       // non-positive std deviation
};

template <typename R>
struct AgProblem {
  int n_cameras, n_instances, n_shots;
  int64_t n_points, n_obs;
  const int32_t* cam_model;
  const R* cam_values;   // [n_cameras][16]
  const R* inst_pose;    // [n_instances][6]
  const R* points;       // [n_points][3]
  const int32_t* shot_inst;
  const int32_t* shot_cam;
  const int32_t* obs_shot;
  const int32_t* obs_point;
  const R* obs_xy;       // [n_obs][2]
  const R* obs_std;      // [n_obs]
};

template <typename R>
AgProblem<R> ag_problem(const gbba_device_problem_t* p) {
  AgProblem<R> a{};
  a.n_cameras = p->n_cameras;
  a.n_instances = p->n_instances;
  a.n_shots = p->n_shots;
  a.n_points = p->n_points;
  a.n_obs = p->n_observations;
  a.cam_model = p->camera_projection;
  a.cam_values = static_cast<const R*>(p->camera_values);
  a.inst_pose = static_cast<const R*>(p->instance_poses);
  a.points = static_cast<const R*>(p->points);
  a.shot_inst = p->shot_instance;
  a.shot_cam = p->shot_camera;
  a.obs_shot = p->obs_shot;
  a.obs_point = p->obs_point;
  a.obs_xy = static_cast<const R*>(p->obs_xy);
  a.obs_std = static_cast<const R*>(p->obs_std);
  return a;
}

__device__ __forceinline__ void ag_report(unsigned long long* st, unsigned long long flag, int64_t index) {
  atomicOr(st, flag);
  atomicMin(st + 1, static_cast<unsigned long long>(index));
}

// Per-shot rotation, right Jacobian and centre (the instance pose is the
// shot pose).  Rejected shots get cam = -1.
template <typename R>
__global__ void ag_shot_kernel(AgProblem<R> a, ShotGeom<R>* geom, unsigned long long* st) {
  const int sh = blockIdx.x * blockDim.x + threadIdx.x;
  if (sh >= a.n_shots) return;
  ShotGeom<R> g{};
  g.cam = R(-1);
  const int ii = a.shot_inst[sh], cam = a.shot_cam[sh];
  if (ii < 0 || ii >= a.n_instances || cam < 0 || cam >= a.n_cameras) {
    ag_report(st, kAgBadShot, sh);
    geom[sh] = g;
    return;
  }
  const int model = a.cam_model[cam];
  if (model < 0 || model >= kNumProjections || model == kSpherical) {
    ag_report(st, kAgBadModel, sh);
    geom[sh] = g;
    return;
  }
  double r[6], Rm[9], Jr[9];
  for (int k = 0; k < 6; ++k) r[k] = double(a.inst_pose[6 * ii + k]);
  pose_rotation(r, Rm, Jr);
  for (int k = 0; k < 9; ++k) {
    g.rot[k] = R(Rm[k]);
    g.jr[k] = R(Jr[k]);
  }
  for (int k = 0; k < 3; ++k) {
    g.tc[k] = R(0);
    g.chi[k] = a.inst_pose[6 * ii + 3 + k];
    g.clo[k] = R(0);
  }
  g.cam = R(cam);
  g.inst = R(ii);
  g.rig = R(-1);
  geom[sh] = g;
}

// Loads one observation's inputs; false if it is invalid (reported once,
// by the forward pass).
template <typename R, int M>
__device__ __forceinline__ bool ag_inputs(const AgProblem<R>& a, const ShotGeom<R>* geom, int64_t i, bool report,
                                          unsigned long long* st, ObsInputs<R>& in, int& sh, int& pt) {
  sh = a.obs_shot[i];
  pt = a.obs_point[i];
  if (sh < 0 || sh >= a.n_shots || pt < 0 || pt >= a.n_points) {
    if (report) ag_report(st, kAgBadObs, i);
    return false;
  }
  const R sd = a.obs_std[i];
  if (!(sd > R(0))) {
    if (report) ag_report(st, kAgBadStd, i);
    return false;
  }
  in.g = geom[sh];
  const int cam = int(in.g.cam);
  if (cam < 0) return false;
  in.ox = a.obs_xy[2 * i];
  in.oy = a.obs_xy[2 * i + 1];
  in.w = R(1) / sd;
  for (int k = 0; k < 3; ++k) in.v[k] = a.points[3 * int64_t(pt) + k] - in.g.chi[k];
  in.rg = nullptr;
  in.cam = a.cam_values + int64_t(cam) * kMaxCameraParams;
  in.model = M >= 0 ? M : a.cam_model[cam];
  return true;
}

// Forward: residuals [n][2]; with records != null also the Jacobian
// records (16-byte planes, plane p of observation i at rec[p * n + i]).
template <typename R, int M, int CMAX>
__global__ void __launch_bounds__(256) ag_forward_kernel(AgProblem<R> a, const ShotGeom<R>* __restrict__ geom,
                                                         R* __restrict__ res, typename Vec16<R>::type* records,
                                                         unsigned long long* st) {
  using L = RecordLayout<2, CMAX, false>;
  constexpr int NP = planes_of<R>(L::kWidth);
  constexpr int VN = Vec16<R>::kN;
  const int64_t stride = int64_t(gridDim.x) * blockDim.x;
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < a.n_obs; i += stride) {
    R rec[NP * VN];
#pragma unroll
    for (int k = 0; k < NP * VN; ++k) rec[k] = R(0);
    ObsInputs<R> in;
    int sh, pt;
    const bool ok = ag_inputs<R, M>(a, geom, i, true, st, in, sh, pt);
    if (ok) {
      if (records) eval_observation<R, M, 2, CMAX, false, true>(in, rec);
      else eval_observation<R, M, 2, CMAX, false, false>(in, rec);
    }
    const R nan = R(0) / R(0);
    res[2 * i] = ok ? rec[L::kR] : nan;
    res[2 * i + 1] = ok ? rec[L::kR + 1] : nan;
    if (records) {
#pragma unroll
      for (int p = 0; p < NP; ++p) store_plane<R>(records + p * a.n_obs + i, rec + p * VN);
    }
  }
}

// Backward: grad_cam[cam][k] += sum J_cam^T g, grad_pose[inst] += J_inst^T g,
// grad_pt[pt] += J_pt^T g, with warp aggregation of equal keys.  Camera
// and pose gradients (few keys shared by many observations) are summed per
// block in shared memory when they fit, and flushed once per block.
constexpr int kAgSharedInst = 512;

template <typename R, int M, int CMAX>
__global__ void __launch_bounds__(256) ag_backward_kernel(AgProblem<R> a, const ShotGeom<R>* __restrict__ geom,
                                                          const R* __restrict__ grad_res,
                                                          const typename Vec16<R>::type* __restrict__ records,
                                                          R* __restrict__ grad_cam, R* __restrict__ grad_pose,
                                                          R* __restrict__ grad_pt) {
  using L = RecordLayout<2, CMAX, false>;
  constexpr int NP = planes_of<R>(L::kWidth);
  constexpr int VN = Vec16<R>::kN;
  __shared__ R s_gc[kSharedCameras * kMaxCameraParams];
  __shared__ R s_gp[kAgSharedInst * 6];
  const bool shared_cam = a.n_cameras <= kSharedCameras;
  const bool shared_pose = a.n_instances <= kAgSharedInst;
  if (grad_cam && shared_cam)
    for (int k = threadIdx.x; k < a.n_cameras * kMaxCameraParams; k += blockDim.x) s_gc[k] = R(0);
  if (grad_pose && shared_pose)
    for (int k = threadIdx.x; k < a.n_instances * 6; k += blockDim.x) s_gp[k] = R(0);
  __syncthreads();
  auto d_cam = [grad_cam](int b, int k) { return grad_cam + int64_t(b) * kMaxCameraParams + k; };
  auto d_pose = [grad_pose](int b, int k) { return grad_pose + 6 * int64_t(b) + k; };
  R* sgc = s_gc;
  R* sgp = s_gp;
  auto s_cam = [sgc](int b, int k) { return sgc + b * kMaxCameraParams + k; };
  auto s_pose = [sgp](int b, int k) { return sgp + 6 * b + k; };
  auto d_pt = [grad_pt](int b, int k) { return grad_pt + 3 * int64_t(b) + k; };
  KeyCarry<CMAX, R, false> c_cam;
  KeyCarry<6, R, false> c_pose;
  KeyCarry<3, R, false> c_pt;
  const int64_t warp0 = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = (int64_t(gridDim.x) * blockDim.x) >> 5;
  const int lane = int(threadIdx.x & 31u);
  for (int64_t base = warp0 * 32; base < a.n_obs; base += nwarps * 32) {
    const int64_t i = base + lane;
    R rec[NP * VN];
#pragma unroll
    for (int k = 0; k < NP * VN; ++k) rec[k] = R(0);
    bool ok = false;
    int sh = 0, pt = 0, cam = -1, inst = -1;
    if (i < a.n_obs) {
      ObsInputs<R> in;
      ok = ag_inputs<R, M>(a, geom, i, false, nullptr, in, sh, pt);
      if (ok) {
        cam = int(in.g.cam);
        inst = int(in.g.inst);
        if (records) load_record<R, NP>(records, a.n_obs, i, rec);
        else eval_observation<R, M, 2, CMAX, false, true>(in, rec);
      }
    }
    const R g0 = ok ? grad_res[2 * i] : R(0), g1 = ok ? grad_res[2 * i + 1] : R(0);
    if (grad_cam) {
      R v[CMAX];
#pragma unroll
      for (int k = 0; k < CMAX; ++k) v[k] = rec[L::kCam + k] * g0 + rec[L::kCam + CMAX + k] * g1;
      if (shared_cam) c_cam.add(ok ? cam : -1, v, s_cam);
      else c_cam.add(ok ? cam : -1, v, d_cam);
    }
    if (grad_pose) {
      R v[6];
#pragma unroll
      for (int k = 0; k < 6; ++k) v[k] = rec[L::kInst + k] * g0 + rec[L::kInst + 6 + k] * g1;
      if (shared_pose) c_pose.add(ok ? inst : -1, v, s_pose);
      else c_pose.add(ok ? inst : -1, v, d_pose);
    }
    if (grad_pt) {
      R v[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) v[k] = rec[L::kPt + k] * g0 + rec[L::kPt + 3 + k] * g1;
      c_pt.add(ok ? pt : -1, v, d_pt);
    }
  }
  __syncthreads();
  if (grad_cam && shared_cam)
    for (int k = threadIdx.x; k < a.n_cameras * kMaxCameraParams; k += blockDim.x)
      if (s_gc[k] != R(0)) red_add(grad_cam + k, s_gc[k]);
  if (grad_pose && shared_pose)
    for (int k = threadIdx.x; k < a.n_instances * 6; k += blockDim.x)
      if (s_gp[k] != R(0)) red_add(grad_pose + k, s_gp[k]);
}

int ag_grid(int64_t n) {
  const int64_t want = (n + 255) / 256;
  return int(want < 1 ? 1 : (want > 152 * 8 ? 152 * 8 : want));
}

// Calls f.template run<M, CMAX>() for the problem's model (a single-model
// hint selects the specialised kernels; -1 the dynamic ones).
template <typename F>
void ag_dispatch(int model, F&& f) {
  switch (model) {
    case kPerspective: f.template run<kPerspective, 3>(); return;
    case kBrown: f.template run<kBrown, 9>(); return;
    case kFisheye: f.template run<kFisheye, 3>(); return;
    case kFisheyeOpencv: f.template run<kFisheyeOpencv, 8>(); return;
    case kFisheye62: f.template run<kFisheye62, 12>(); return;
    case kFisheye624: f.template run<kFisheye624, 16>(); return;
    case kDual: f.template run<kDual, 4>(); return;
    case kRadial: f.template run<kRadial, 6>(); return;
    case kSimpleRadial: f.template run<kSimpleRadial, 5>(); return;
    default: f.template run<kAgDyn, 16>(); return;
  }
}

int ag_cmax(int model) {
  if (model >= 0 && model < kNumProjections && model != kSpherical) return model_num_params(model);
  return kMaxCameraParams;
}

void ag_check(const gbba_device_problem_t* p) {
  if (!p) throw ApiError(GBBA_ERR_INVALID_ARGUMENT, "problem is NULL");
  if (p->dtype != GBBA_DTYPE_F64 && p->dtype != GBBA_DTYPE_F32)
    throw ApiError(GBBA_ERR_INVALID_ARGUMENT, "dtype must be GBBA_DTYPE_F64 or GBBA_DTYPE_F32");
  if (p->n_cameras < 0 || p->n_instances < 0 || p->n_shots < 0 || p->n_points < 0 || p->n_observations < 0)
    throw ApiError(GBBA_ERR_INVALID_ARGUMENT, "negative count in problem");
  if (p->model_hint == kSpherical)
    throw ApiError(GBBA_ERR_INVALID_ARGUMENT, "spherical cameras are not supported by the projection operator");
  if (p->model_hint < -1 || p->model_hint >= kNumProjections)
    throw ApiError(GBBA_ERR_INVALID_ARGUMENT, "unknown model hint");
}

size_t ag_geom_bytes(const gbba_device_problem_t* p) {
  const size_t g = p->dtype == GBBA_DTYPE_F64 ? sizeof(ShotGeom<double>) : sizeof(ShotGeom<float>);
  return g * size_t(p->n_shots > 0 ? p->n_shots : 1);
}

template <typename R>
struct AgForward {
  AgProblem<R> a;
  ShotGeom<R>* geom;
  R* res;
  typename Vec16<R>::type* records;
  unsigned long long* st;
  cudaStream_t s;
  template <int M, int CMAX>
  void run() {
    ag_forward_kernel<R, M, CMAX><<<ag_grid(a.n_obs), 256, 0, s>>>(a, geom, res, records, st);
  }
};

template <typename R>
struct AgBackward {
  AgProblem<R> a;
  const ShotGeom<R>* geom;
  const R* grad_res;
  const typename Vec16<R>::type* records;
  R *gc, *gp, *gx;
  cudaStream_t s;
  template <int M, int CMAX>
  void run() {
    // fewer, longer-lived blocks: each flushes its shared camera / pose sums once
    const int64_t want = (a.n_obs + 255) / 256;
    const int grid = int(want < 1 ? 1 : (want > 152 * 4 ? 152 * 4 : want));
    ag_backward_kernel<R, M, CMAX><<<grid, 256, 0, s>>>(a, geom, grad_res, records, gc, gp, gx);
  }
};

template <typename R>
void ag_forward(const gbba_device_problem_t* p, void* residuals, void* records, void* scratch, cudaStream_t s) {
  AgProblem<R> a = ag_problem<R>(p);
  auto* base = static_cast<unsigned char*>(scratch);
  auto* st = reinterpret_cast<unsigned long long*>(base);
  auto* geom = reinterpret_cast<ShotGeom<R>*>(base + kAgStatusBytes);
  GB_CUDA(cudaMemsetAsync(st, 0, sizeof(unsigned long long), s));
  GB_CUDA(cudaMemsetAsync(st + 1, 0xff, sizeof(unsigned long long), s));
  if (a.n_shots > 0) ag_shot_kernel<R><<<(a.n_shots + 127) / 128, 128, 0, s>>>(a, geom, st);
  if (a.n_obs > 0) {
    AgForward<R> f{a, geom, static_cast<R*>(residuals), static_cast<typename Vec16<R>::type*>(records), st, s};
    ag_dispatch(p->model_hint, f);
  }
  GB_CUDA(cudaGetLastError());
  unsigned long long h[2] = {0, 0};
  GB_CUDA(cudaMemcpyAsync(h, st, sizeof(h), cudaMemcpyDeviceToHost, s));
  GB_CUDA(cudaStreamSynchronize(s));
  if (h[0] & kAgBadShot) throw ApiError(GBBA_ERR_OUT_OF_RANGE, "shot " + std::to_string(h[1]) + " references a missing block");
  if (h[0] & kAgBadModel)
    throw ApiError(GBBA_ERR_INVALID_ARGUMENT, "shot " + std::to_string(h[1]) + ": unknown or spherical camera model");
  if (h[0] & kAgBadObs)
    throw ApiError(GBBA_ERR_OUT_OF_RANGE, "observation " + std::to_string(h[1]) + " references a missing shot or point");
  if (h[0] & kAgBadStd)
    throw ApiError(GBBA_ERR_INVALID_ARGUMENT, "observation " + std::to_string(h[1]) + " has non-positive std");
}

template <typename R>
void ag_backward(const gbba_device_problem_t* p, const void* grad_res, const void* records, void* gc, void* gp,
                 void* gx, const void* scratch, cudaStream_t s) {
  AgProblem<R> a = ag_problem<R>(p);
  auto* geom = reinterpret_cast<const ShotGeom<R>*>(static_cast<const unsigned char*>(scratch) + kAgStatusBytes);
  if (a.n_obs > 0) {
    AgBackward<R> f{a, geom, static_cast<const R*>(grad_res), static_cast<const typename Vec16<R>::type*>(records),
                    static_cast<R*>(gc), static_cast<R*>(gp), static_cast<R*>(gx), s};
    ag_dispatch(p->model_hint, f);
  }
  GB_CUDA(cudaGetLastError());
}

}  // namespace
}  // namespace gbba

using gbba::ApiError;

extern "C" {

int gbba_projection_scratch_bytes(const gbba_device_problem_t* p, int64_t* bytes) {
  return gbba::guarded([&] {
    gbba::ag_check(p);
    if (!bytes) throw ApiError(GBBA_ERR_INVALID_ARGUMENT, "bytes is NULL");
    *bytes = int64_t(gbba::kAgStatusBytes + gbba::ag_geom_bytes(p));
  });
}

int gbba_projection_record_bytes(const gbba_device_problem_t* p, int64_t* bytes) {
  return gbba::guarded([&] {
    gbba::ag_check(p);
    if (!bytes) throw ApiError(GBBA_ERR_INVALID_ARGUMENT, "bytes is NULL");
    const int cmax = gbba::ag_cmax(p->model_hint);
    const int width = 2 + 3 * 2 + 6 * 2 + cmax * 2;
    const int planes = p->dtype == GBBA_DTYPE_F64 ? (width + 1) / 2 : (width + 3) / 4;
    *bytes = int64_t(planes) * 16 * p->n_observations;
  });
}

int gbba_projection_forward(const gbba_device_problem_t* p, void* residuals, void* records, void* scratch,
                            void* stream) {
  return gbba::guarded([&] {
    gbba::ag_check(p);
    if (!residuals || !scratch) throw ApiError(GBBA_ERR_INVALID_ARGUMENT, "residuals or scratch is NULL");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (p->dtype == GBBA_DTYPE_F64) gbba::ag_forward<double>(p, residuals, records, scratch, s);
    else gbba::ag_forward<float>(p, residuals, records, scratch, s);
  });
}

int gbba_projection_backward(const gbba_device_problem_t* p, const void* grad_residuals, const void* records,
                             const void* scratch, void* grad_camera_values, void* grad_instance_poses,
                             void* grad_points, void* stream) {
  return gbba::guarded([&] {
    gbba::ag_check(p);
    if (!grad_residuals || !scratch) throw ApiError(GBBA_ERR_INVALID_ARGUMENT, "grad_residuals or scratch is NULL");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (p->dtype == GBBA_DTYPE_F64)
      gbba::ag_backward<double>(p, grad_residuals, records, grad_camera_values, grad_instance_poses, grad_points,
                                scratch, s);
    else
      gbba::ag_backward<float>(p, grad_residuals, records, grad_camera_values, grad_instance_poses, grad_points,
                               scratch, s);
  });
}

}  // extern "C"
