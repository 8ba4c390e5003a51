// Residual + Jacobian evaluation that allocates no memory
// (gbba_evaluate_projections_noalloc).
//
// Who needs it.  gbba_evaluate_projections copies the scene to the device
// and allocates its intermediates on every call.  Some callers cannot
// allocate at the moment they evaluate: a serving process that has carved
// all of the device's memory into its own pool up front (a cudaMalloc would
// fail, or would grow and fragment the footprint it budgeted), a real-time
// loop where an allocation's implicit synchronisation would stall the
// device, or a host runtime whose device memory comes from its own
// allocator.  Such a caller already holds the scene and the output arrays in
// device memory it owns; this entry point evaluates straight from them and
// keeps its one intermediate -- the per-shot geometry (rotation, rotation
// derivative, centre) -- in a fixed file-scope device array.
//
// Limits and rules:
//   - at most kNoAllocMaxShots shots; larger scenes are rejected with
//     GBBA_ERR_INVALID_ARGUMENT (use gbba_evaluate_projections);
//   - FP64 arithmetic (the same per-observation math as the FP64 path of
//     gbba_evaluate_projections);
//   - the scratch is one array per device for the whole process: calls that
//     overlap on the same device (from two threads, or on two streams
//     without ordering) race on it and must be serialised by the caller;
//   - the first call on a device (with that device current) looks up the
//     scratch's device address; that lookup may load the library's device
//     code, so make the first call before any stream capture on that device;
//   - the call waits for its stream to finish before it returns, because it
//     reads back the status word the kernels write.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>
#include <string>

#include "../../include/gbba.h"
#include "capi_util.h"
#include "eval_kernels.cuh"

namespace gbba {
namespace {

constexpr int kNoAllocMaxShots = 8192;
constexpr int kNoAllocMaxDevices = 64;
constexpr int kDynModel = -1;

// Status words written by the kernels (the scratch's first 64 bytes):
//   [0] flags, [1] first bad shot, [2] first bad observation.
enum : unsigned long long {
  kBadShot = 1,        // a shot references a missing instance / camera / rig camera
  kBadModel = 2,       // a camera's projection type is unknown
  kBadObsIndex = 4,    // an observation references a missing shot or point
  kBadStd = 8,         // an observation's std deviation is not positive
  kBadWidth = 16,      // cmax_out or nr too small for a camera of the scene
};
constexpr size_t kStatusBytes = 256;
constexpr size_t kGeomBytes = sizeof(ShotGeom<double>) * kNoAllocMaxShots;
constexpr size_t kRigBytes = sizeof(RigGeom<double>) * kNoAllocMaxShots;
constexpr size_t kScratchBytes = kStatusBytes + kGeomBytes + kRigBytes;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

struct DevScene {
  int n_cameras, n_instances, n_rig_cameras, n_shots;
  int64_t n_points, n_obs;
  int nr_out, cmax_out;
  const int32_t* cam_model;
  const double* cam_values;
  const double* inst_pose;
  const double* rig_pose;
  const uint8_t* rig_used;  // may be null: no rig camera applied
  const int32_t* shot_inst;
  const int32_t* shot_rig;
  const int32_t* shot_cam;
  const double* points;
  const int32_t* obs_shot;
  const int32_t* obs_point;
  const double* obs_xy;
  const double* obs_std;
};

__device__ __forceinline__ void report(unsigned long long* st, unsigned long long flag, int slot, long long index) {
  atomicOr(st, flag);
  atomicMin(st + slot, static_cast<unsigned long long>(index));
}

// Per-shot geometry with every index checked first.  Same composition as
// shot_prep_kernel (instance pose, then the rig-camera pose); a rejected
// shot is stored with cam = -1 so that its observations are skipped.
__global__ void noalloc_shot_kernel(DevScene s, ShotGeom<double>* geom, RigGeom<double>* rig,
                                    unsigned long long* st) {
  const int sh = blockIdx.x * blockDim.x + threadIdx.x;
  if (sh >= s.n_shots) return;
  const int ii = s.shot_inst[sh], rc = s.shot_rig[sh], cam = s.shot_cam[sh];
  ShotGeom<double> g{};
  g.cam = -1.0;
  if (ii < 0 || ii >= s.n_instances || cam < 0 || cam >= s.n_cameras || rc < -1 || rc >= s.n_rig_cameras) {
    report(st, kBadShot, 1, sh);
    geom[sh] = g;
    return;
  }
  const int model = s.cam_model[cam];
  if (model < 0 || model >= kNumProjections) {
    report(st, kBadModel, 1, sh);
    geom[sh] = g;
    return;
  }
  const double* pi = s.inst_pose + 6 * ii;
  double Ri[9], Ji[9];
  pose_rotation(pi, Ri, Ji);
  const bool use_rig = rc >= 0 && s.rig_used != nullptr && s.rig_used[rc] != 0;
  double rot[9], tc[3] = {0.0, 0.0, 0.0};
  double Rr[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1}, Jr[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1}, cr[3] = {0.0, 0.0, 0.0};
  if (use_rig) {
    const double* pr = s.rig_pose + 6 * rc;
    pose_rotation(pr, Rr, Jr);
    for (int k = 0; k < 3; ++k) cr[k] = pr[3 + k];
    for (int m = 0; m < 3; ++m) {
      for (int j = 0; j < 3; ++j) {
        double a = 0.0;
        for (int n = 0; n < 3; ++n) a += Rr[m * 3 + n] * Ri[n * 3 + j];
        rot[m * 3 + j] = a;
      }
      tc[m] = -(Rr[m * 3 + 0] * cr[0] + Rr[m * 3 + 1] * cr[1] + Rr[m * 3 + 2] * cr[2]);
    }
  } else {
    for (int k = 0; k < 9; ++k) rot[k] = Ri[k];
  }
  for (int k = 0; k < 9; ++k) {
    g.rot[k] = rot[k];
    g.jr[k] = Ji[k];
  }
  for (int k = 0; k < 3; ++k) {
    g.tc[k] = tc[k];
    g.chi[k] = pi[3 + k];
    g.clo[k] = 0.0;
  }
  g.cam = double(cam);
  g.inst = double(ii);
  g.rig = use_rig ? double(rc) : -1.0;
  geom[sh] = g;
  RigGeom<double> q{};
  for (int k = 0; k < 9; ++k) {
    q.rinst[k] = Ri[k];
    q.rrc[k] = Rr[k];
    q.jrc[k] = Jr[k];
  }
  for (int k = 0; k < 3; ++k) q.crc[k] = cr[k];
  rig[sh] = q;
}

// One observation per thread: residual and Jacobian blocks written straight
// into the caller's arrays (the layout gbba_evaluate_projections returns).
template <int NR, bool RIG>
__global__ void __launch_bounds__(256) noalloc_eval_kernel(DevScene s, const ShotGeom<double>* __restrict__ geom,
                                                           const RigGeom<double>* __restrict__ rig,
                                                           gbba_eval_output_t o, unsigned long long* st) {
  using L = RecordLayout<NR, kMaxCameraParams, RIG>;
  const int64_t stride = int64_t(gridDim.x) * blockDim.x;
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < s.n_obs; i += stride) {
    double rec[L::kWidth];
#pragma unroll
    for (int k = 0; k < L::kWidth; ++k) rec[k] = 0.0;
    const int sh = s.obs_shot[i], pt = s.obs_point[i];
    const double sd = s.obs_std[i];
    if (sh < 0 || sh >= s.n_shots || pt < 0 || pt >= s.n_points) {
      report(st, kBadObsIndex, 2, i);
    } else if (!(sd > 0.0)) {
      report(st, kBadStd, 2, i);
    } else {
      ObsInputs<double> in;
      in.g = geom[sh];
      const int cam = int(in.g.cam);
      if (cam >= 0) {
        const int model = s.cam_model[cam];
        if (model_num_params(model) > s.cmax_out || (NR == 2 && model == kSpherical)) {
          report(st, kBadWidth, 2, i);
        } else {
          in.ox = s.obs_xy[2 * i];
          in.oy = s.obs_xy[2 * i + 1];
          in.w = 1.0 / sd;
          for (int k = 0; k < 3; ++k) in.v[k] = s.points[3 * int64_t(pt) + k] - in.g.chi[k];
          in.rg = RIG ? rig + sh : nullptr;
          in.cam = s.cam_values + int64_t(cam) * kMaxCameraParams;
          in.model = model;
          eval_observation<double, kDynModel, NR, kMaxCameraParams, RIG, true>(in, rec);
        }
      }
    }
    const int nr = s.nr_out, co = s.cmax_out;
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      if (r >= nr) break;
      const bool row = r < NR;
      const int rr = row ? r : 0;  // keeps every record index in range
      const int64_t ir = i * nr + r;
      if (o.residuals) o.residuals[ir] = row ? rec[L::kR + rr] : 0.0;
      if (o.jac_point) {
#pragma unroll
        for (int j = 0; j < 3; ++j) o.jac_point[ir * 3 + j] = row ? rec[L::kPt + rr * 3 + j] : 0.0;
      }
      if (o.jac_instance) {
#pragma unroll
        for (int j = 0; j < 6; ++j) o.jac_instance[ir * 6 + j] = row ? rec[L::kInst + rr * 6 + j] : 0.0;
      }
      if (o.jac_rig_camera) {
#pragma unroll
        for (int j = 0; j < 6; ++j)
          o.jac_rig_camera[ir * 6 + j] = (row && RIG) ? rec[(RIG ? L::kRig : 0) + rr * 6 + j] : 0.0;
      }
      if (o.jac_camera) {
#pragma unroll
        for (int j = 0; j < kMaxCameraParams; ++j)
          if (j < co) o.jac_camera[ir * co + j] = row ? rec[L::kCam + rr * kMaxCameraParams + j] : 0.0;
      }
    }
  }
}

// Device address of the scratch, looked up once per device.
void* scratch_address(int device) {
  static std::mutex mu;
  static void* addr[kNoAllocMaxDevices] = {};
  if (device < 0 || device >= kNoAllocMaxDevices)
    throw ApiError(GBBA_ERR_INVALID_ARGUMENT, "device ordinal out of range");
  std::lock_guard<std::mutex> lock(mu);
  if (!addr[device]) {
    void* p = nullptr;
    GB_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    addr[device] = p;
  }
  return addr[device];
}

// Rejects pointers the kernels could not dereference (host memory): the
// kernels would fault on them.
void require_device(const void* p, const char* what, int device) {
  if (!p) throw ApiError(GBBA_ERR_INVALID_ARGUMENT, std::string(what) + " is NULL");
  cudaPointerAttributes a{};
  GB_CUDA(cudaPointerGetAttributes(&a, p));
  const bool ok = (a.type == cudaMemoryTypeDevice && a.device == device) || a.type == cudaMemoryTypeManaged;
  if (!ok) throw ApiError(GBBA_ERR_INVALID_ARGUMENT, std::string(what) + " is not device memory of the current device");
}

int grid_of(int64_t n) {
  const int64_t want = (n + 255) / 256;
  return int(want < 1 ? 1 : (want > 152 * 8 ? 152 * 8 : want));
}

}  // namespace
}  // namespace gbba

using gbba::ApiError;

extern "C" int gbba_evaluate_projections_noalloc(const gbba_scene_t* scene, int nr, int cmax_out,
                                                 gbba_eval_output_t* out, void* stream) {
  using namespace gbba;
  return guarded([&] {
    if (!scene || !out) throw ApiError(GBBA_ERR_INVALID_ARGUMENT, "scene or output is NULL");
    if (nr != 2 && nr != 3) throw ApiError(GBBA_ERR_INVALID_ARGUMENT, "nr must be 2 or 3");
    if (cmax_out < 1 || cmax_out > kMaxCameraParams)
      throw ApiError(GBBA_ERR_INVALID_ARGUMENT, "cmax_out must be in [1, 16]");
    if (scene->n_cameras < 0 || scene->n_rig_instances < 0 || scene->n_rig_cameras < 0 || scene->n_shots < 0 ||
        scene->n_points < 0 || scene->n_observations < 0)
      throw ApiError(GBBA_ERR_INVALID_ARGUMENT, "negative count in scene");
    if (scene->n_shots > kNoAllocMaxShots)
      throw ApiError(GBBA_ERR_INVALID_ARGUMENT, "scene has " + std::to_string(scene->n_shots) +
                                                    " shots; gbba_evaluate_projections_noalloc supports at most " +
                                                    std::to_string(kNoAllocMaxShots));
    if (scene->n_observations == 0) return;
    int device = 0;
    GB_CUDA(cudaGetDevice(&device));
    const bool rigs = scene->n_rig_cameras > 0;
    require_device(scene->camera_projection, "camera_projection", device);
    require_device(scene->camera_values, "camera_values", device);
    require_device(scene->rig_instance_poses, "rig_instance_poses", device);
    if (rigs) require_device(scene->rig_camera_poses, "rig_camera_poses", device);
    if (rigs && scene->rig_camera_used) require_device(scene->rig_camera_used, "rig_camera_used", device);
    require_device(scene->shot_rig_instance, "shot_rig_instance", device);
    require_device(scene->shot_rig_camera, "shot_rig_camera", device);
    require_device(scene->shot_camera, "shot_camera", device);
    require_device(scene->points, "points", device);
    require_device(scene->obs_shot, "obs_shot", device);
    require_device(scene->obs_point, "obs_point", device);
    require_device(scene->obs_xy, "obs_xy", device);
    require_device(scene->obs_std, "obs_std", device);
    const char* names[5] = {"residuals", "jac_camera", "jac_instance", "jac_rig_camera", "jac_point"};
    double* outs[5] = {out->residuals, out->jac_camera, out->jac_instance, out->jac_rig_camera, out->jac_point};
    for (int k = 0; k < 5; ++k)
      if (outs[k]) require_device(outs[k], names[k], device);

    unsigned char* base = static_cast<unsigned char*>(scratch_address(device));
    auto* status = reinterpret_cast<unsigned long long*>(base);
    auto* geom = reinterpret_cast<ShotGeom<double>*>(base + kStatusBytes);
    auto* rig = reinterpret_cast<RigGeom<double>*>(base + kStatusBytes + kGeomBytes);
    cudaStream_t st = static_cast<cudaStream_t>(stream);

    DevScene s{};
    s.n_cameras = scene->n_cameras;
    s.n_instances = scene->n_rig_instances;
    s.n_rig_cameras = scene->n_rig_cameras;
    s.n_shots = scene->n_shots;
    s.n_points = scene->n_points;
    s.n_obs = scene->n_observations;
    s.nr_out = nr;
    s.cmax_out = cmax_out;
    s.cam_model = scene->camera_projection;
    s.cam_values = scene->camera_values;
    s.inst_pose = scene->rig_instance_poses;
    s.rig_pose = rigs ? scene->rig_camera_poses : nullptr;
    s.rig_used = rigs ? scene->rig_camera_used : nullptr;
    s.shot_inst = scene->shot_rig_instance;
    s.shot_rig = scene->shot_rig_camera;
    s.shot_cam = scene->shot_camera;
    s.points = scene->points;
    s.obs_shot = scene->obs_shot;
    s.obs_point = scene->obs_point;
    s.obs_xy = scene->obs_xy;
    s.obs_std = scene->obs_std;

    // status: flags start at zero, first-bad indices at the maximum
    GB_CUDA(cudaMemsetAsync(status, 0, sizeof(unsigned long long), st));
    GB_CUDA(cudaMemsetAsync(status + 1, 0xff, 2 * sizeof(unsigned long long), st));
    if (s.n_shots > 0) {
      noalloc_shot_kernel<<<(s.n_shots + 127) / 128, 128, 0, st>>>(s, geom, rig, status);
      GB_CUDA(cudaGetLastError());
    }
    const int g = grid_of(s.n_obs);
    if (nr == 2) {
      if (rigs) noalloc_eval_kernel<2, true><<<g, 256, 0, st>>>(s, geom, rig, *out, status);
      else noalloc_eval_kernel<2, false><<<g, 256, 0, st>>>(s, geom, rig, *out, status);
    } else {
      if (rigs) noalloc_eval_kernel<3, true><<<g, 256, 0, st>>>(s, geom, rig, *out, status);
      else noalloc_eval_kernel<3, false><<<g, 256, 0, st>>>(s, geom, rig, *out, status);
    }
    GB_CUDA(cudaGetLastError());
    unsigned long long h[3] = {0, 0, 0};
    GB_CUDA(cudaMemcpyAsync(h, status, sizeof(h), cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaStreamSynchronize(st));
    if (h[0] & (kBadShot | kBadModel)) {
      const std::string what = (h[0] & kBadModel) ? "has an invalid ProjectionType" : "references a missing block";
      throw ApiError((h[0] & kBadModel) ? GBBA_ERR_RUNTIME : GBBA_ERR_OUT_OF_RANGE,
                     "shot " + std::to_string(h[1]) + " " + what);
    }
    if (h[0] & kBadObsIndex)
      throw ApiError(GBBA_ERR_OUT_OF_RANGE,
                     "observation " + std::to_string(h[2]) + " references a missing shot or point");
    if (h[0] & kBadStd)
      throw ApiError(GBBA_ERR_INVALID_ARGUMENT, "observation " + std::to_string(h[2]) + " has non-positive std");
    if (h[0] & kBadWidth)
      throw ApiError(GBBA_ERR_INVALID_ARGUMENT, "observation " + std::to_string(h[2]) +
                                                    ": nr or cmax_out is smaller than its camera needs");
  });
}
