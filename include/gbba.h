/*
 * gbba.h -- C ABI of the GB300 bundle adjuster.
 *
 * A drop-in for the bundle adjuster of OpenSfM (opensfm/src/lib/bundle):
 * the C++ class bundle::BundleAdjuster (bundle_adjuster.h:173-386) and its
 * pybind module opensfm.pybundle (python/pybind.cc:60-147).  Every entry
 * point takes plain pointers and sizes, never throws, and returns a status
 * code; the message of the last failure is available from
 * gbba_last_error().
 *
 * Camera model ids follow geometry::ProjectionType
 * (opensfm/src/lib/geometry/camera_instances.h:8-20) and camera parameter
 * vectors follow the order of geometry::Camera
 * (opensfm/src/lib/geometry/src/camera.cc:11-172).  Poses are
 * camera-to-world [rx, ry, rz, tx, ty, tz] (angle-axis, camera centre) as in
 * bundle::Pose (opensfm/src/lib/bundle/data/pose.h:17,34-43).
 */
#ifndef GBBA_H_
#define GBBA_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes.  GBBA_ERR_RUNTIME corresponds to std::runtime_error in the
 * reference (unknown camera / rig / point ids, unknown loss or linear solver,
 * non-finite depth prior); GBBA_ERR_OUT_OF_RANGE to std::out_of_range from
 * std::map::at (unknown shot or point in
 * AddPointProjectionObservation, bundle_adjuster.cc:274-287). */
enum {
  GBBA_OK = 0,
  GBBA_ERR_INVALID_ARGUMENT = 1,
  GBBA_ERR_RUNTIME = 2,
  GBBA_ERR_OUT_OF_RANGE = 3,
  GBBA_ERR_CUDA = 4,
  GBBA_ERR_INTERNAL = 5
};

/* Camera models (geometry::ProjectionType order). */
enum {
  GBBA_PERSPECTIVE = 0,
  GBBA_BROWN = 1,
  GBBA_FISHEYE = 2,
  GBBA_FISHEYE_OPENCV = 3,
  GBBA_FISHEYE62 = 4,
  GBBA_FISHEYE624 = 5,
  GBBA_SPHERICAL = 6,
  GBBA_DUAL = 7,
  GBBA_RADIAL = 8,
  GBBA_SIMPLE_RADIAL = 9
};

/* Arithmetic of the device path. */
enum { GBBA_PRECISION_FP64 = 0, GBBA_PRECISION_MIXED = 1 };

/* Maximum number of intrinsic parameters of a camera (FISHEYE624). */
#define GBBA_MAX_CAMERA_PARAMS 16

/* Number of intrinsic parameters of a camera model, or -1 if unknown. */
int gbba_camera_num_params(int projection);

/* Message of the last error raised on this thread ("" if none). */
const char* gbba_last_error(void);

/* ------------------------------------------------------------------------
 * Batched residual + Jacobian evaluation.
 *
 * The batched equivalent of ReprojectionError2DAnalytic<C>::Evaluate and
 * ReprojectionError3DAnalytic::Evaluate
 * (opensfm/src/lib/bundle/error/projection_errors.h:67-207, :255-374) over
 * every observation of a scene.  A scene is given as flat host arrays.
 */
typedef struct gbba_scene {
  int32_t n_cameras;
  const int32_t* camera_projection; /* [n_cameras] model id */
  const double* camera_values;      /* [n_cameras][GBBA_MAX_CAMERA_PARAMS] */
  int32_t n_rig_instances;
  const double* rig_instance_poses; /* [n_rig_instances][6] */
  int32_t n_rig_cameras;
  const double* rig_camera_poses;   /* [n_rig_cameras][6] */
  const uint8_t* rig_camera_used;   /* [n_rig_cameras] 0: identity, not applied */
  int32_t n_shots;
  const int32_t* shot_rig_instance; /* [n_shots] */
  const int32_t* shot_rig_camera;   /* [n_shots] */
  const int32_t* shot_camera;       /* [n_shots] */
  int64_t n_points;
  const double* points;             /* [n_points][3] */
  int64_t n_observations;
  const int32_t* obs_shot;          /* [n_observations] */
  const int32_t* obs_point;         /* [n_observations] */
  const double* obs_xy;             /* [n_observations][2] normalized coords */
  const double* obs_std;            /* [n_observations] std deviation */
} gbba_scene_t;

/* Output buffers of an evaluation, all row-major FP64, one block per
 * observation:  residuals [nr], jac_camera [nr][cmax], jac_instance [nr][6],
 * jac_rig_camera [nr][6], jac_point [nr][3].  nr is 3 when the scene holds a
 * spherical camera, else 2; cmax is the largest parameter count among the
 * scene's camera models.  Any Jacobian pointer may be NULL to skip it. */
typedef struct gbba_eval_output {
  double* residuals;
  double* jac_camera;
  double* jac_instance;
  double* jac_rig_camera;
  double* jac_point;
} gbba_eval_output_t;

/* Layout of the evaluation outputs for a scene (nr and cmax above). */
int gbba_scene_layout(const gbba_scene_t* scene, int* nr, int* cmax);

/* One-shot evaluation from host buffers: upload, evaluate on the GPU,
 * download.  precision is GBBA_PRECISION_FP64 or GBBA_PRECISION_MIXED. */
int gbba_evaluate_projections(const gbba_scene_t* scene, int precision,
                              gbba_eval_output_t* out);

/* Device-resident evaluator: the scene is uploaded once, evaluations run on
 * the device (stream is a cudaStream_t, NULL for the default stream). */
typedef struct gbba_evaluator gbba_evaluator_t;
gbba_evaluator_t* gbba_evaluator_create(const gbba_scene_t* scene, int precision);
void gbba_evaluator_destroy(gbba_evaluator_t* ev);
int gbba_evaluator_run(gbba_evaluator_t* ev, void* stream);
/* The two halves of gbba_evaluator_run: the per-shot pose precompute and the
 * per-observation residual/Jacobian record kernel (for timing each alone). */
int gbba_evaluator_prepare(gbba_evaluator_t* ev, void* stream);
int gbba_evaluator_records(gbba_evaluator_t* ev, void* stream);
int gbba_evaluator_download(gbba_evaluator_t* ev, gbba_eval_output_t* out);
/* Number of kernel launches of one gbba_evaluator_run call. */
int gbba_evaluator_launches_per_run(const gbba_evaluator_t* ev);
/* Bytes of the device-side residual+Jacobian records of one run. */
int64_t gbba_evaluator_record_bytes(const gbba_evaluator_t* ev);

#ifdef __cplusplus
}
#endif

#endif /* GBBA_H_ */
