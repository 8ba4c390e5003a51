// Standalone batched residual + Jacobian evaluation behind the C ABI
// (gbba_evaluate_projections / gbba_evaluator_*).  This is the GPU
// counterpart of calling ReprojectionError2DAnalytic<C>::Evaluate
// (opensfm/src/lib/bundle/error/projection_errors.h:67-207) for every
// observation of a problem.
#include <algorithm>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "../../include/gbba.h"
#include "capi_util.h"
#include "device_buffer.h"
#include "eval_kernels.cuh"

namespace gbba {

namespace {

constexpr int kDynamicModel = -1;

// Conversion of device records to the reference's per-block FP64 layout.
template <typename R, int NR, int CMAX, bool RIG>
__global__ void records_to_blocks_kernel(int64_t n, const typename Vec16<R>::type* __restrict__ rec_planes,
                                         int64_t plane_stride, int nr_out, int cmax_out,
                                         double* __restrict__ res, double* __restrict__ jc,
                                         double* __restrict__ ji, double* __restrict__ jr,
                                         double* __restrict__ jp) {
  using L = RecordLayout<NR, CMAX, RIG>;
  constexpr int NP = planes_of<R>(L::kWidth);
  constexpr int VN = Vec16<R>::kN;
  const int64_t stride = int64_t(gridDim.x) * blockDim.x;
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) {
    R rec[NP * VN];
#pragma unroll
    for (int p = 0; p < NP; ++p) load_plane<R>(rec_planes + p * plane_stride + i, rec + p * VN);
    for (int r = 0; r < nr_out; ++r) {
      const bool row = r < NR;
      res[i * nr_out + r] = row ? double(rec[L::kR + r]) : 0.0;
      if (jp)
        for (int j = 0; j < 3; ++j) jp[(i * nr_out + r) * 3 + j] = row ? double(rec[L::kPt + r * 3 + j]) : 0.0;
      if (ji)
        for (int j = 0; j < 6; ++j) ji[(i * nr_out + r) * 6 + j] = row ? double(rec[L::kInst + r * 6 + j]) : 0.0;
      if (jr)
        for (int j = 0; j < 6; ++j)
          jr[(i * nr_out + r) * 6 + j] = (row && RIG) ? double(rec[(RIG ? L::kRig : 0) + r * 6 + j]) : 0.0;
      if (jc)
        for (int j = 0; j < cmax_out; ++j)
          jc[(i * nr_out + r) * cmax_out + j] = (row && j < CMAX) ? double(rec[L::kCam + r * CMAX + j]) : 0.0;
    }
  }
}

// ---------------------------------------------------------------------------
// Direct evaluation for devices that read and write pageable host memory
// (GB300 next to a Grace CPU: address translation over NVLink-C2C).  The
// one-shot entry point then streams the caller's observation arrays into
// the kernel and writes the FP64 blocks straight into the caller's output
// arrays: no staging copies, no device-side records.  Observation indices
// and std deviations are checked in the kernel; a bad one is recorded in
// `status` (flags, first bad observation) and its outputs are zeros.
enum : unsigned long long { kDirectBadIndex = 1, kDirectBadStd = 2 };

struct DirectObs {
  int64_t n;
  int32_t n_shots;
  int64_t n_points;
  const int32_t* shot;
  const int32_t* point;
  const double* xy;
  const double* std_dev;
};

template <typename R>
__global__ void convert_points_kernel(int64_t n, const double* __restrict__ xyz,
                                      typename PointStore<R>::type* __restrict__ out) {
  const int64_t stride = int64_t(gridDim.x) * blockDim.x;
  for (int64_t p = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; p < n; p += stride)
    out[p] = make_point_store(xyz[3 * p], xyz[3 * p + 1], xyz[3 * p + 2], static_cast<R*>(nullptr));
}

// Per-warp staging of one output array: every lane puts its observation's
// NR x width block into shared memory, then the warp writes the 32
// observations' contiguous range with consecutive lanes on consecutive
// doubles (whole-line writes over the CPU link instead of strided ones).
__device__ __forceinline__ void flush_staged(double* __restrict__ dst, const double* __restrict__ buf, int64_t first,
                                             int per_obs, int count) {
  __syncwarp();
  double* base = dst + first * per_obs;
  const int total = count * per_obs;
  for (int k = int(threadIdx.x & 31u); k < total; k += 32) base[k] = buf[k];
  __syncwarp();
}

constexpr int kDirectBlock = 128;

template <int NR, int CMAX>
constexpr int direct_stage_doubles() {
  return 32 * NR * (CMAX > 6 ? CMAX : 6);
}

template <typename R, int M, int NR, int CMAX, bool RIG>
__global__ void __launch_bounds__(kDirectBlock) direct_eval_kernel(SceneView<R> s, DirectObs d, gbba_eval_output_t o,
                                                                   int cmax_out,
                                                                   unsigned long long* __restrict__ status) {
  using L = RecordLayout<NR, CMAX, RIG>;
  __shared__ R s_cam[kSharedCameras * kMaxCameraParams];
  __shared__ int s_model[kSharedCameras];
  extern __shared__ double s_stage[];
  const int* models;
  const R* cams = stage_cameras(s, s_cam, s_model, models);
  const int lane = int(threadIdx.x & 31u);
  double* buf = s_stage + (threadIdx.x >> 5) * direct_stage_doubles<NR, CMAX>();
  const int64_t warp0 = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = (int64_t(gridDim.x) * blockDim.x) >> 5;
  for (int64_t first = warp0 * 32; first < d.n; first += nwarps * 32) {
    const int64_t i = first + lane;
    const int count = int(d.n - first < 32 ? d.n - first : 32);
    R rec[L::kWidth];
#pragma unroll
    for (int k = 0; k < L::kWidth; ++k) rec[k] = R(0);
    if (i < d.n) {
      const int sh = d.shot[i], pt = d.point[i];
      const double sd = d.std_dev[i];
      if (sh < 0 || sh >= d.n_shots || pt < 0 || pt >= d.n_points) {
        atomicOr(status, kDirectBadIndex);
        atomicMin(status + 1, static_cast<unsigned long long>(i));
      } else if (!(sd > 0.0)) {
        atomicOr(status, kDirectBadStd);
        atomicMin(status + 1, static_cast<unsigned long long>(i));
      } else {
        ObsPack<R> ob{};
        ob.x = R(d.xy[2 * i]);
        ob.y = R(d.xy[2 * i + 1]);
        ob.w = R(1.0 / sd);
        ob.shot = sh;
        ObsInputs<R> in;
        load_inputs<R, M>(s, ob, pt, cams, models, in);
        eval_observation<R, M, NR, CMAX, RIG, true>(in, rec);
      }
    }
    if (o.residuals) {
#pragma unroll
      for (int r = 0; r < NR; ++r) buf[lane * NR + r] = double(rec[L::kR + r]);
      flush_staged(o.residuals, buf, first, NR, count);
    }
    if (o.jac_point) {
#pragma unroll
      for (int r = 0; r < NR; ++r)
#pragma unroll
        for (int j = 0; j < 3; ++j) buf[(lane * NR + r) * 3 + j] = double(rec[L::kPt + r * 3 + j]);
      flush_staged(o.jac_point, buf, first, NR * 3, count);
    }
    if (o.jac_instance) {
#pragma unroll
      for (int r = 0; r < NR; ++r)
#pragma unroll
        for (int j = 0; j < 6; ++j) buf[(lane * NR + r) * 6 + j] = double(rec[L::kInst + r * 6 + j]);
      flush_staged(o.jac_instance, buf, first, NR * 6, count);
    }
    if (o.jac_rig_camera) {
#pragma unroll
      for (int r = 0; r < NR; ++r)
#pragma unroll
        for (int j = 0; j < 6; ++j)
          buf[(lane * NR + r) * 6 + j] = RIG ? double(rec[(RIG ? L::kRig : 0) + r * 6 + j]) : 0.0;
      flush_staged(o.jac_rig_camera, buf, first, NR * 6, count);
    }
    if (o.jac_camera) {
#pragma unroll
      for (int r = 0; r < NR; ++r)
#pragma unroll
        for (int j = 0; j < CMAX; ++j)
          if (j < cmax_out) buf[(lane * NR + r) * cmax_out + j] = double(rec[L::kCam + r * CMAX + j]);
      flush_staged(o.jac_camera, buf, first, NR * cmax_out, count);
    }
  }
}

int grid_for(int64_t n, int block) {
  const int64_t want = (n + block - 1) / block;
  const int64_t cap = 152 * 16;
  return int(std::max<int64_t>(1, std::min(want, cap)));
}

struct Layout {
  int model;  // single model id, or kDynamicModel
  int nr;
  int cmax;   // record columns of the camera block
  bool rig;
  int cmax_out;
};

template <typename R>
struct EvalState {
  using PS = typename PointStore<R>::type;
  DeviceArray<ShotGeom<R>> geom;
  DeviceArray<RigGeom<R>> rig;
  DeviceArray<int> shot_cam, cam_model, shot_inst, shot_rig;
  DeviceArray<R> cam_params;
  DeviceArray<double> inst_pose, rig_pose;
  DeviceArray<uint8_t> rig_used;
  DeviceArray<PS> points;
  DeviceArray<ObsPack<R>> obs;
  DeviceArray<int> obs_point;
  DeviceArray<typename Vec16<R>::type> records;
  int64_t n_obs = 0;
  int n_shots = 0;
  int n_cameras = 0;
  int n_planes = 0;

  SceneView<R> view() const {
    SceneView<R> v;
    v.n_slots = n_obs;
    v.n_cameras = n_cameras;
    v.geom = geom.get();
    v.rig = rig.size() ? rig.get() : nullptr;

    v.cam_model = cam_model.get();
    v.cam_params = cam_params.get();
    v.points = points.get();
    v.obs = obs.get();
    v.obs_point = obs_point.get();
    return v;
  }
};

// Instantiation table of the record kernel.
template <typename R, int M, int NR, int CMAX, bool RIG>
void launch_eval(const SceneView<R>& v, typename Vec16<R>::type* out, int64_t stride, cudaStream_t st) {
  eval_records_kernel<R, M, NR, CMAX, RIG><<<grid_for(v.n_slots, 256), 256, 0, st>>>(v, out, stride, ~uint64_t(0));
}
template <typename R, int NR, int CMAX, bool RIG>
void launch_blocks(int64_t n, const typename Vec16<R>::type* rec, int64_t stride, int nr_out, int cmax_out,
                   double* res, double* jc, double* ji, double* jr, double* jp, cudaStream_t st) {
  records_to_blocks_kernel<R, NR, CMAX, RIG>
      <<<grid_for(n, 256), 256, 0, st>>>(n, rec, stride, nr_out, cmax_out, res, jc, ji, jr, jp);
}

template <typename R>
void dispatch_eval(const Layout& L, const SceneView<R>& v, typename Vec16<R>::type* out, int64_t stride,
                   cudaStream_t st) {
  if (L.model != kDynamicModel) {
    switch (L.model) {
      case kPerspective: launch_eval<R, kPerspective, 2, 3, false>(v, out, stride, st); return;
      case kBrown: launch_eval<R, kBrown, 2, 9, false>(v, out, stride, st); return;
      case kFisheye: launch_eval<R, kFisheye, 2, 3, false>(v, out, stride, st); return;
      case kFisheyeOpencv: launch_eval<R, kFisheyeOpencv, 2, 8, false>(v, out, stride, st); return;
      case kFisheye62: launch_eval<R, kFisheye62, 2, 12, false>(v, out, stride, st); return;
      case kFisheye624: launch_eval<R, kFisheye624, 2, 16, false>(v, out, stride, st); return;
      case kDual: launch_eval<R, kDual, 2, 4, false>(v, out, stride, st); return;
      case kRadial: launch_eval<R, kRadial, 2, 6, false>(v, out, stride, st); return;
      case kSimpleRadial: launch_eval<R, kSimpleRadial, 2, 5, false>(v, out, stride, st); return;
    }
  }
  if (L.nr == 2) {
    if (L.rig) launch_eval<R, kDynamicModel, 2, 16, true>(v, out, stride, st);
    else launch_eval<R, kDynamicModel, 2, 16, false>(v, out, stride, st);
  } else {
    if (L.rig) launch_eval<R, kDynamicModel, 3, 16, true>(v, out, stride, st);
    else launch_eval<R, kDynamicModel, 3, 16, false>(v, out, stride, st);
  }
}

template <typename R>
void dispatch_blocks(const Layout& L, int64_t n, const typename Vec16<R>::type* rec, int64_t stride,
                     const gbba_eval_output_t& o, cudaStream_t st) {
  double *res = o.residuals, *jc = o.jac_camera, *ji = o.jac_instance, *jr = o.jac_rig_camera,
         *jp = o.jac_point;
  const int nr = L.nr, co = L.cmax_out;
  if (L.model != kDynamicModel) {
    switch (L.cmax) {
      case 3: launch_blocks<R, 2, 3, false>(n, rec, stride, nr, co, res, jc, ji, jr, jp, st); return;
      case 4: launch_blocks<R, 2, 4, false>(n, rec, stride, nr, co, res, jc, ji, jr, jp, st); return;
      case 5: launch_blocks<R, 2, 5, false>(n, rec, stride, nr, co, res, jc, ji, jr, jp, st); return;
      case 6: launch_blocks<R, 2, 6, false>(n, rec, stride, nr, co, res, jc, ji, jr, jp, st); return;
      case 8: launch_blocks<R, 2, 8, false>(n, rec, stride, nr, co, res, jc, ji, jr, jp, st); return;
      case 9: launch_blocks<R, 2, 9, false>(n, rec, stride, nr, co, res, jc, ji, jr, jp, st); return;
      case 12: launch_blocks<R, 2, 12, false>(n, rec, stride, nr, co, res, jc, ji, jr, jp, st); return;
      case 16: launch_blocks<R, 2, 16, false>(n, rec, stride, nr, co, res, jc, ji, jr, jp, st); return;
    }
  }
  if (L.nr == 2) {
    if (L.rig) launch_blocks<R, 2, 16, true>(n, rec, stride, nr, co, res, jc, ji, jr, jp, st);
    else launch_blocks<R, 2, 16, false>(n, rec, stride, nr, co, res, jc, ji, jr, jp, st);
  } else {
    if (L.rig) launch_blocks<R, 3, 16, true>(n, rec, stride, nr, co, res, jc, ji, jr, jp, st);
    else launch_blocks<R, 3, 16, false>(n, rec, stride, nr, co, res, jc, ji, jr, jp, st);
  }
}

template <int NR, int CMAX, bool RIG>
int record_width() {
  return RecordLayout<NR, CMAX, RIG>::kWidth;
}

int layout_width(const Layout& L) {
  if (L.model != kDynamicModel) return RecordLayout<2, 1, false>::kCam + 2 * L.cmax;
  const int base = L.nr + 3 * L.nr + 6 * L.nr + 16 * L.nr;
  return base + (L.rig ? 6 * L.nr : 0);
}

template <typename R, int M, int NR, int CMAX, bool RIG>
void launch_direct(const SceneView<R>& v, const DirectObs& d, const gbba_eval_output_t& o, int nr_out,
                   int cmax_out, unsigned long long* status) {
  if (nr_out != NR || cmax_out > CMAX) throw std::logic_error("direct evaluation layout mismatch");
  auto* k = direct_eval_kernel<R, M, NR, CMAX, RIG>;
  const int smem = int(sizeof(double)) * direct_stage_doubles<NR, CMAX>() * (kDirectBlock / 32);
  GB_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  k<<<grid_for(d.n, kDirectBlock), kDirectBlock, smem>>>(v, d, o, cmax_out, status);
}

template <typename R>
void dispatch_direct(const Layout& L, const SceneView<R>& v, const DirectObs& d, const gbba_eval_output_t& o,
                     unsigned long long* status) {
  const int nr = L.nr, co = L.cmax_out;
  if (L.model != kDynamicModel) {
    switch (L.model) {
      case kPerspective: launch_direct<R, kPerspective, 2, 3, false>(v, d, o, nr, co, status); return;
      case kBrown: launch_direct<R, kBrown, 2, 9, false>(v, d, o, nr, co, status); return;
      case kFisheye: launch_direct<R, kFisheye, 2, 3, false>(v, d, o, nr, co, status); return;
      case kFisheyeOpencv: launch_direct<R, kFisheyeOpencv, 2, 8, false>(v, d, o, nr, co, status); return;
      case kFisheye62: launch_direct<R, kFisheye62, 2, 12, false>(v, d, o, nr, co, status); return;
      case kFisheye624: launch_direct<R, kFisheye624, 2, 16, false>(v, d, o, nr, co, status); return;
      case kDual: launch_direct<R, kDual, 2, 4, false>(v, d, o, nr, co, status); return;
      case kRadial: launch_direct<R, kRadial, 2, 6, false>(v, d, o, nr, co, status); return;
      case kSimpleRadial: launch_direct<R, kSimpleRadial, 2, 5, false>(v, d, o, nr, co, status); return;
    }
  }
  if (L.nr == 2) {
    if (L.rig) launch_direct<R, kDynamicModel, 2, 16, true>(v, d, o, nr, co, status);
    else launch_direct<R, kDynamicModel, 2, 16, false>(v, d, o, nr, co, status);
  } else {
    if (L.rig) launch_direct<R, kDynamicModel, 3, 16, true>(v, d, o, nr, co, status);
    else launch_direct<R, kDynamicModel, 3, 16, false>(v, d, o, nr, co, status);
  }
}

bool device_reads_host_memory() {
  int dev = 0, v = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return false;
  if (cudaDeviceGetAttribute(&v, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess) return false;
  return v != 0;
}

// Counts, camera models and shot references (small arrays, checked on the
// host before anything is launched).
void validate_scene_blocks(const gbba_scene_t* s) {
  if (!s) throw ApiError(GBBA_ERR_INVALID_ARGUMENT, "scene is NULL");
  if (s->n_cameras < 0 || s->n_rig_instances < 0 || s->n_rig_cameras < 0 || s->n_shots < 0 ||
      s->n_points < 0 || s->n_observations < 0)
    throw ApiError(GBBA_ERR_INVALID_ARGUMENT, "negative count in scene");
  for (int c = 0; c < s->n_cameras; ++c) {
    const int m = s->camera_projection[c];
    if (m < 0 || m >= kNumProjections)
      throw ApiError(GBBA_ERR_RUNTIME, "Invalid ProjectionType for camera " + std::to_string(c));
  }
  for (int i = 0; i < s->n_shots; ++i) {
    if (s->shot_rig_instance[i] < 0 || s->shot_rig_instance[i] >= s->n_rig_instances ||
        s->shot_camera[i] < 0 || s->shot_camera[i] >= s->n_cameras ||
        s->shot_rig_camera[i] < -1 || s->shot_rig_camera[i] >= s->n_rig_cameras)
      throw ApiError(GBBA_ERR_OUT_OF_RANGE, "shot " + std::to_string(i) + " references a missing block");
  }
}

void validate_scene(const gbba_scene_t* s) {
  if (!s) throw ApiError(GBBA_ERR_INVALID_ARGUMENT, "scene is NULL");
  if (s->n_cameras < 0 || s->n_rig_instances < 0 || s->n_rig_cameras < 0 || s->n_shots < 0 ||
      s->n_points < 0 || s->n_observations < 0)
    throw ApiError(GBBA_ERR_INVALID_ARGUMENT, "negative count in scene");
  for (int c = 0; c < s->n_cameras; ++c) {
    const int m = s->camera_projection[c];
    if (m < 0 || m >= kNumProjections)
      throw ApiError(GBBA_ERR_RUNTIME, "Invalid ProjectionType for camera " + std::to_string(c));
  }
  for (int i = 0; i < s->n_shots; ++i) {
    if (s->shot_rig_instance[i] < 0 || s->shot_rig_instance[i] >= s->n_rig_instances ||
        s->shot_camera[i] < 0 || s->shot_camera[i] >= s->n_cameras ||
        s->shot_rig_camera[i] < -1 || s->shot_rig_camera[i] >= s->n_rig_cameras)
      throw ApiError(GBBA_ERR_OUT_OF_RANGE, "shot " + std::to_string(i) + " references a missing block");
  }
  for (int64_t i = 0; i < s->n_observations; ++i) {
    if (s->obs_shot[i] < 0 || s->obs_shot[i] >= s->n_shots || s->obs_point[i] < 0 ||
        s->obs_point[i] >= s->n_points)
      throw ApiError(GBBA_ERR_OUT_OF_RANGE, "observation " + std::to_string(i) + " references a missing shot or point");
    if (!(s->obs_std[i] > 0.0))
      throw ApiError(GBBA_ERR_INVALID_ARGUMENT, "observation " + std::to_string(i) + " has non-positive std");
  }
}

Layout scene_layout(const gbba_scene_t* s) {
  Layout L;
  bool any_sph = false, any_rig = false;
  int cmax = 1, first = -1;
  bool single = true;
  std::vector<uint8_t> cam_used(s->n_cameras, 0);
  for (int i = 0; i < s->n_shots; ++i) {
    cam_used[s->shot_camera[i]] = 1;
    const int rc = s->shot_rig_camera[i];
    if (rc >= 0 && s->rig_camera_used && s->rig_camera_used[rc]) any_rig = true;
  }
  for (int c = 0; c < s->n_cameras; ++c) {
    if (!cam_used[c]) continue;
    const int m = s->camera_projection[c];
    if (m == kSpherical) any_sph = true;
    cmax = std::max(cmax, model_num_params(m));
    if (first < 0) first = m;
    else if (first != m) single = false;
  }
  L.nr = any_sph ? 3 : 2;
  L.rig = any_rig;
  L.cmax_out = cmax;
  if (single && !any_sph && !any_rig && first >= 0) {
    L.model = first;
    L.cmax = model_num_params(first);
  } else {
    L.model = kDynamicModel;
    L.cmax = 16;
  }
  return L;
}

// One-shot evaluation reading the scene's arrays and writing the output
// arrays in place (device_reads_host_memory() must hold).  Only the small
// per-camera / per-shot tables and the points (converted to the working
// precision) are staged in device memory.
template <typename R>
void evaluate_direct(const gbba_scene_t* s, const Layout& L, gbba_eval_output_t* out) {
  using PS = typename PointStore<R>::type;
  const int ns = s->n_shots;
  DeviceArray<R> cam_params;
  DeviceArray<int> cam_model, shot_inst, shot_rig, shot_cam;
  DeviceArray<double> inst_pose, rig_pose;
  DeviceArray<uint8_t> rig_used;
  DeviceArray<ShotGeom<R>> geom(std::max(1, ns));
  DeviceArray<RigGeom<R>> rig;
  DeviceArray<PS> points(std::max<int64_t>(1, s->n_points));
  DeviceArray<unsigned long long> status(2);
  {
    std::vector<R> cam(size_t(s->n_cameras) * kMaxCameraParams);
    for (size_t i = 0; i < cam.size(); ++i) cam[i] = R(s->camera_values[i]);
    cam_params.upload(cam);
  }
  cam_model.upload(s->camera_projection, s->n_cameras);
  shot_cam.upload(s->shot_camera, ns);
  shot_inst.upload(s->shot_rig_instance, ns);
  shot_rig.upload(s->shot_rig_camera, ns);
  inst_pose.upload(s->rig_instance_poses, size_t(s->n_rig_instances) * 6);
  {
    std::vector<double> rp(size_t(std::max(1, s->n_rig_cameras)) * 6, 0.0);
    std::vector<uint8_t> ru(size_t(std::max(1, s->n_rig_cameras)), 0);
    for (int i = 0; i < s->n_rig_cameras; ++i) {
      for (int k = 0; k < 6; ++k) rp[i * 6 + k] = s->rig_camera_poses[i * 6 + k];
      ru[i] = s->rig_camera_used ? s->rig_camera_used[i] : 0;
    }
    rig_pose.upload(rp);
    rig_used.upload(ru);
  }
  if (L.rig) rig.resize(std::max(1, ns));
  GB_CUDA(cudaMemset(status.get(), 0, sizeof(unsigned long long)));
  GB_CUDA(cudaMemset(status.get() + 1, 0xff, sizeof(unsigned long long)));
  if (s->n_points > 0) {
    convert_points_kernel<R><<<grid_for(s->n_points, 256), 256>>>(s->n_points, s->points, points.get());
    GB_CUDA(cudaGetLastError());
  }
  if (ns > 0) {
    shot_prep_kernel<R><<<(ns + 127) / 128, 128>>>(ns, shot_inst.get(), shot_rig.get(), shot_cam.get(),
                                                   inst_pose.get(), rig_pose.get(), rig_used.get(), geom.get(),
                                                   L.rig ? rig.get() : nullptr);
    GB_CUDA(cudaGetLastError());
  }
  SceneView<R> v{};
  v.n_slots = s->n_observations;
  v.n_cameras = s->n_cameras;
  v.geom = geom.get();
  v.rig = L.rig ? rig.get() : nullptr;
  v.cam_model = cam_model.get();
  v.cam_params = cam_params.get();
  v.points = points.get();
  DirectObs d{s->n_observations, s->n_shots, s->n_points, s->obs_shot, s->obs_point, s->obs_xy, s->obs_std};
  dispatch_direct<R>(L, v, d, *out, status.get());
  GB_CUDA(cudaGetLastError());
  unsigned long long h[2] = {0, 0};
  GB_CUDA(cudaMemcpy(h, status.get(), sizeof(h), cudaMemcpyDeviceToHost));
  if (h[0] & kDirectBadIndex)
    throw ApiError(GBBA_ERR_OUT_OF_RANGE, "observation " + std::to_string(h[1]) + " references a missing shot or point");
  if (h[0] & kDirectBadStd)
    throw ApiError(GBBA_ERR_INVALID_ARGUMENT, "observation " + std::to_string(h[1]) + " has non-positive std");
}

}  // namespace

// Holds a device-resident scene in one precision.
struct EvaluatorImpl {
  int precision = GBBA_PRECISION_MIXED;
  Layout L{};
  EvalState<float> f;
  EvalState<double> d;

  template <typename R>
  EvalState<R>& st();

  template <typename R>
  void upload(const gbba_scene_t* s) {
    EvalState<R>& e = st<R>();
    e.n_obs = s->n_observations;
    e.n_shots = s->n_shots;
    std::vector<R> cam(size_t(s->n_cameras) * kMaxCameraParams);
    for (size_t i = 0; i < cam.size(); ++i) cam[i] = R(s->camera_values[i]);
    e.cam_params.upload(cam);
    e.cam_model.upload(s->camera_projection, s->n_cameras);
    e.shot_cam.upload(s->shot_camera, s->n_shots);
    e.shot_inst.upload(s->shot_rig_instance, s->n_shots);
    e.shot_rig.upload(s->shot_rig_camera, s->n_shots);
    e.inst_pose.upload(s->rig_instance_poses, size_t(s->n_rig_instances) * 6);
    std::vector<double> rp(size_t(std::max(1, s->n_rig_cameras)) * 6, 0.0);
    std::vector<uint8_t> ru(size_t(std::max(1, s->n_rig_cameras)), 0);
    for (int i = 0; i < s->n_rig_cameras; ++i) {
      for (int k = 0; k < 6; ++k) rp[i * 6 + k] = s->rig_camera_poses[i * 6 + k];
      ru[i] = s->rig_camera_used ? s->rig_camera_used[i] : 0;
    }
    e.rig_pose.upload(rp);
    e.rig_used.upload(ru);
    using PS = typename PointStore<R>::type;
    std::vector<PS> pts(size_t(s->n_points));
    for (int64_t i = 0; i < s->n_points; ++i)
      pts[i] = make_point_store(s->points[3 * i], s->points[3 * i + 1], s->points[3 * i + 2],
                                static_cast<R*>(nullptr));
    e.points.upload(pts);
    e.obs_point.upload(s->obs_point, size_t(s->n_observations));
    std::vector<ObsPack<R>> ob(size_t(s->n_observations));
    for (int64_t i = 0; i < s->n_observations; ++i) {
      ob[i].x = R(s->obs_xy[2 * i]);
      ob[i].y = R(s->obs_xy[2 * i + 1]);
      ob[i].w = R(1.0 / s->obs_std[i]);
      ob[i].shot = s->obs_shot[i];
    }
    e.obs.upload(ob);
    e.n_cameras = s->n_cameras;
    e.geom.resize(std::max(1, s->n_shots));

    if (L.rig) e.rig.resize(std::max(1, s->n_shots));
    e.n_planes = planes_of<R>(layout_width(L));
    e.records.resize(size_t(e.n_planes) * std::max<int64_t>(1, e.n_obs));
    GB_CUDA(cudaStreamSynchronize(0));
  }

  template <typename R>
  void run(cudaStream_t stream) {
    prepare<R>(stream);
    records<R>(stream);
  }

  template <typename R>
  void prepare(cudaStream_t stream) {
    EvalState<R>& e = st<R>();
    if (e.n_shots > 0) {
      shot_prep_kernel<R><<<(e.n_shots + 127) / 128, 128, 0, stream>>>(
          e.n_shots, e.shot_inst.get(), e.shot_rig.get(), e.shot_cam.get(), e.inst_pose.get(), e.rig_pose.get(),
          e.rig_used.get(), e.geom.get(), L.rig ? e.rig.get() : nullptr);
      GB_CUDA(cudaGetLastError());
    }
  }

  template <typename R>
  void records(cudaStream_t stream) {
    EvalState<R>& e = st<R>();
    if (e.n_obs > 0) {
      dispatch_eval<R>(L, e.view(), e.records.get(), e.n_obs, stream);
      GB_CUDA(cudaGetLastError());
    }
  }

  template <typename R>
  void download(gbba_eval_output_t* out) {
    EvalState<R>& e = st<R>();
    const int64_t n = e.n_obs;
    if (n == 0) return;
    const int nr = L.nr, co = L.cmax_out;
    DeviceArray<double> res(size_t(n) * nr), jc, ji, jr, jp;
    if (out->jac_camera) jc.resize(size_t(n) * nr * co);
    if (out->jac_instance) ji.resize(size_t(n) * nr * 6);
    if (out->jac_rig_camera) jr.resize(size_t(n) * nr * 6);
    if (out->jac_point) jp.resize(size_t(n) * nr * 3);
    gbba_eval_output_t dev{res.get(), jc.size() ? jc.get() : nullptr, ji.size() ? ji.get() : nullptr,
                           jr.size() ? jr.get() : nullptr, jp.size() ? jp.get() : nullptr};
    dispatch_blocks<R>(L, n, e.records.get(), n, dev, 0);
    GB_CUDA(cudaGetLastError());
    if (out->residuals) res.download(out->residuals, res.size());
    if (out->jac_camera) jc.download(out->jac_camera, jc.size());
    if (out->jac_instance) ji.download(out->jac_instance, ji.size());
    if (out->jac_rig_camera) jr.download(out->jac_rig_camera, jr.size());
    if (out->jac_point) jp.download(out->jac_point, jp.size());
    GB_CUDA(cudaStreamSynchronize(0));
  }

  int64_t record_bytes() const {
    return precision == GBBA_PRECISION_FP64 ? int64_t(d.n_planes) * 16 * d.n_obs
                                            : int64_t(f.n_planes) * 16 * f.n_obs;
  }
};
template <> EvalState<float>& EvaluatorImpl::st<float>() { return f; }
template <> EvalState<double>& EvaluatorImpl::st<double>() { return d; }

}  // namespace gbba

struct gbba_evaluator {
  gbba::EvaluatorImpl impl;
};

using gbba::ApiError;

extern "C" {

int gbba_camera_num_params(int projection) {
  if (projection < 0 || projection >= gbba::kNumProjections) return -1;
  return gbba::model_num_params(projection);
}

int gbba_scene_layout(const gbba_scene_t* scene, int* nr, int* cmax) {
  return gbba::guarded([&] {
    gbba::validate_scene(scene);
    const gbba::Layout L = gbba::scene_layout(scene);
    if (nr) *nr = L.nr;
    if (cmax) *cmax = L.cmax_out;
  });
}

gbba_evaluator_t* gbba_evaluator_create(const gbba_scene_t* scene, int precision) {
  gbba_evaluator_t* ev = nullptr;
  const int st = gbba::guarded([&] {
    if (precision != GBBA_PRECISION_FP64 && precision != GBBA_PRECISION_MIXED)
      throw ApiError(GBBA_ERR_INVALID_ARGUMENT, "unknown precision");
    gbba::validate_scene(scene);
    std::unique_ptr<gbba_evaluator_t> e(new gbba_evaluator_t);
    e->impl.precision = precision;
    e->impl.L = gbba::scene_layout(scene);
    if (precision == GBBA_PRECISION_FP64) e->impl.upload<double>(scene);
    else e->impl.upload<float>(scene);
    ev = e.release();
  });
  return st == GBBA_OK ? ev : nullptr;
}

void gbba_evaluator_destroy(gbba_evaluator_t* ev) { delete ev; }

int gbba_evaluator_run(gbba_evaluator_t* ev, void* stream) {
  return gbba::guarded([&] {
    if (!ev) throw ApiError(GBBA_ERR_INVALID_ARGUMENT, "evaluator is NULL");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (ev->impl.precision == GBBA_PRECISION_FP64) ev->impl.run<double>(s);
    else ev->impl.run<float>(s);
  });
}

int gbba_evaluator_prepare(gbba_evaluator_t* ev, void* stream) {
  return gbba::guarded([&] {
    if (!ev) throw ApiError(GBBA_ERR_INVALID_ARGUMENT, "evaluator is NULL");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (ev->impl.precision == GBBA_PRECISION_FP64) ev->impl.prepare<double>(s);
    else ev->impl.prepare<float>(s);
  });
}

int gbba_evaluator_records(gbba_evaluator_t* ev, void* stream) {
  return gbba::guarded([&] {
    if (!ev) throw ApiError(GBBA_ERR_INVALID_ARGUMENT, "evaluator is NULL");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (ev->impl.precision == GBBA_PRECISION_FP64) ev->impl.records<double>(s);
    else ev->impl.records<float>(s);
  });
}

int gbba_evaluator_download(gbba_evaluator_t* ev, gbba_eval_output_t* out) {
  return gbba::guarded([&] {
    if (!ev || !out) throw ApiError(GBBA_ERR_INVALID_ARGUMENT, "NULL argument");
    GB_CUDA(cudaDeviceSynchronize());
    if (ev->impl.precision == GBBA_PRECISION_FP64) ev->impl.download<double>(out);
    else ev->impl.download<float>(out);
  });
}

int gbba_evaluator_launches_per_run(const gbba_evaluator_t* ev) {
  if (!ev) return 0;
  const int64_t n = ev->impl.precision == GBBA_PRECISION_FP64 ? ev->impl.d.n_obs : ev->impl.f.n_obs;
  const int shots = ev->impl.precision == GBBA_PRECISION_FP64 ? ev->impl.d.n_shots : ev->impl.f.n_shots;
  return (shots > 0 ? 1 : 0) + (n > 0 ? 1 : 0);
}

int64_t gbba_evaluator_record_bytes(const gbba_evaluator_t* ev) { return ev ? ev->impl.record_bytes() : 0; }

int gbba_evaluate_projections(const gbba_scene_t* scene, int precision, gbba_eval_output_t* out) {
  return gbba::guarded([&] {
    if (!out) throw ApiError(GBBA_ERR_INVALID_ARGUMENT, "output is NULL");
    if (precision != GBBA_PRECISION_FP64 && precision != GBBA_PRECISION_MIXED)
      throw ApiError(GBBA_ERR_INVALID_ARGUMENT, "unknown precision");
    if (gbba::device_reads_host_memory()) {
      // the kernels read the caller's arrays and write its outputs in place
      gbba::validate_scene_blocks(scene);
      if (scene->n_observations == 0) return;
      const gbba::Layout L = gbba::scene_layout(scene);
      if (precision == GBBA_PRECISION_FP64) gbba::evaluate_direct<double>(scene, L, out);
      else gbba::evaluate_direct<float>(scene, L, out);
      return;
    }
    gbba_evaluator_t* ev = gbba_evaluator_create(scene, precision);
    if (!ev) throw ApiError(gbba::last_status(), gbba_last_error());
    std::unique_ptr<gbba_evaluator_t, void (*)(gbba_evaluator_t*)> hold(ev, gbba_evaluator_destroy);
    if (gbba_evaluator_run(ev, nullptr) != GBBA_OK) throw ApiError(gbba::last_status(), gbba_last_error());
    if (gbba_evaluator_download(ev, out) != GBBA_OK) throw ApiError(gbba::last_status(), gbba_last_error());
  });
}

}  // extern "C"
