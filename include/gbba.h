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

/* One-shot evaluation from host buffers.  precision is GBBA_PRECISION_FP64
 * or GBBA_PRECISION_MIXED.  Where the GPU reads and writes pageable host
 * memory directly (a GB300 next to a Grace CPU), the kernels stream the
 * observation arrays and write the output arrays in place; elsewhere the
 * scene is uploaded and the blocks downloaded.  An observation with a bad
 * index or a non-positive std returns an error status; the output arrays
 * are then unspecified. */
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

/* Evaluation that allocates no memory.  No counterpart in the reference.
 *
 * For callers that cannot allocate device memory when they evaluate (a
 * process whose device memory is all carved into its own pool, a real-time
 * loop that must not stall on an allocation): every array of `scene` and of
 * `out` is DEVICE memory of the current device, owned by the caller and
 * sized as for gbba_evaluate_projections; the counts in `scene` are host
 * values.  nr and cmax_out give the output layout (gbba_scene_layout on a
 * host copy of the scene returns them).  FP64 arithmetic, the same as
 * gbba_evaluate_projections with GBBA_PRECISION_FP64.  The per-shot geometry
 * lives in a fixed device array of the library:
 *   - at most 8192 shots (more: GBBA_ERR_INVALID_ARGUMENT);
 *   - calls that overlap on one device race on that array: serialise them;
 *   - the first call on a device looks the array up (this may load the
 *     library's device code): make it before any stream capture there.
 * stream is a cudaStream_t (NULL: default stream); the call returns after
 * the stream has finished the evaluation.  Bad indices, unknown projection
 * types and non-positive std deviations are found on the device and
 * returned as the same status codes gbba_evaluate_projections uses. */
int gbba_evaluate_projections_noalloc(const gbba_scene_t* scene, int nr, int cmax_out,
                                      gbba_eval_output_t* out, void* stream);

/* ------------------------------------------------------------------------
 * Differentiable projection + residual (an autograd operator).
 *
 * Forward: r_i = (pi(camera, pose, X) - obs_i) / std_i for every
 * observation, as ReprojectionError2DAnalytic<C>::Evaluate
 * (projection_errors.h:67-207) with the shot pose equal to its rig
 * instance's (no rig camera).  Backward: J^T g for an incoming gradient g
 * of the residuals, added into the gradients of the camera parameter
 * vectors, the instance poses [rx ry rz tx ty tz] and the points.  All
 * arrays are device memory of the caller; every floating array has the
 * problem's dtype.  Spherical cameras are not supported (3-row residual).
 */
enum { GBBA_DTYPE_F64 = 0, GBBA_DTYPE_F32 = 1 };

typedef struct gbba_device_problem {
  int32_t dtype;                     /* GBBA_DTYPE_F64 or GBBA_DTYPE_F32 */
  int32_t model_hint;                /* the single camera model of the problem, or -1 (mixed models) */
  int32_t n_cameras;
  const int32_t* camera_projection;  /* [n_cameras] */
  const void* camera_values;         /* [n_cameras][GBBA_MAX_CAMERA_PARAMS] */
  int32_t n_instances;
  const void* instance_poses;        /* [n_instances][6] */
  int64_t n_points;
  const void* points;                /* [n_points][3] */
  int32_t n_shots;
  const int32_t* shot_instance;      /* [n_shots] */
  const int32_t* shot_camera;        /* [n_shots] */
  int64_t n_observations;
  const int32_t* obs_shot;           /* [n_observations] */
  const int32_t* obs_point;          /* [n_observations] */
  const void* obs_xy;                /* [n_observations][2] */
  const void* obs_std;               /* [n_observations] */
} gbba_device_problem_t;

/* Bytes of the scratch the forward pass fills (per-shot geometry) and the
 * backward pass reads; of the Jacobian records saved by a storing forward. */
int gbba_projection_scratch_bytes(const gbba_device_problem_t* p, int64_t* bytes);
int gbba_projection_record_bytes(const gbba_device_problem_t* p, int64_t* bytes);
/* residuals [n_observations][2]; records NULL to keep no Jacobian (the
 * backward then recomputes it).  Validates every index on the device and
 * waits for the stream; invalid observations get NaN residuals. */
int gbba_projection_forward(const gbba_device_problem_t* p, void* residuals, void* records, void* scratch,
                            void* stream);
/* Any gradient pointer may be NULL; the others are accumulated into. */
int gbba_projection_backward(const gbba_device_problem_t* p, const void* grad_residuals, const void* records,
                             const void* scratch, void* grad_camera_values, void* grad_instance_poses,
                             void* grad_points, void* stream);

/* ------------------------------------------------------------------------
 * Bundle adjuster: bundle::BundleAdjuster (bundle_adjuster.h:173-386) and
 * the methods its pybind module binds (python/pybind.cc:60-147).  Ids are
 * NUL-terminated strings.  Unknown ids raise GBBA_ERR_RUNTIME (the
 * reference's std::runtime_error) except in
 * gbba_add_point_projection_observation, where an unknown shot or point is
 * GBBA_ERR_OUT_OF_RANGE (std::map::at, bundle_adjuster.cc:279-281).
 */
typedef struct gbba_adjuster gbba_adjuster_t;

/* BundleAdjuster::BundleAdjuster (bundle_adjuster.cc:56-75). */
gbba_adjuster_t* gbba_create(void);
void gbba_destroy(gbba_adjuster_t* h);

/* AddCamera (bundle_adjuster.cc:107-129): values and prior_values hold the
 * geometry::Camera parameter vectors; constant fixes every parameter. */
int gbba_add_camera(gbba_adjuster_t* h, const char* id, int projection, const double* values,
                    const double* prior_values, int n_values, int constant);
/* SetCameraBias (bundle_adjuster.cc:131-140): similarity applied to the GPS
 * priors of instances whose reference camera is camera_id
 * (SimilarityPriorTransform, bias.h:34-54: prior -> scale R(rotation) prior
 * + translation).  Its parameters stay fixed unless
 * gbba_set_camera_bias_parameters names some. */
int gbba_set_camera_bias(gbba_adjuster_t* h, const char* camera_id, const double* rotation,
                         const double* translation, double scale);
/* SetCameraBias's parameters_to_optimize (bundle_adjuster.cc:131-140,
 * pybind.cc:68-70): indices of Similarity::Parameter (0-2 rotation, 3-5
 * translation, 6 scale; bias.h:12), n = 0 to hold the bias fixed.  The GPS
 * priors of the instances referencing the camera then optimise the bias
 * with the poses (DataPriorError with SimilarityPriorTransform,
 * bundle_adjuster.cc:806-838); gbba_get_bias reads the solved bias. */
int gbba_set_camera_bias_parameters(gbba_adjuster_t* h, const char* camera_id, const int* indices, int n);
/* GetBias (bundle_adjuster.cc:1317-1323): rotation[3] (angle-axis),
 * translation[3], scale. */
int gbba_get_bias(const gbba_adjuster_t* h, const char* camera_id, double* rotation, double* translation,
                  double* scale);
/* AddRigCamera (bundle_adjuster.cc:179-198). */
int gbba_add_rig_camera(gbba_adjuster_t* h, const char* id, const double* pose, const double* pose_prior,
                        int fixed);
/* AddRigInstance (bundle_adjuster.cc:142-177): creates one shot per entry
 * of (shot_ids, camera_ids, rig_camera_ids). */
int gbba_add_rig_instance(gbba_adjuster_t* h, const char* id, const double* pose, int n_shots,
                          const char* const* shot_ids, const char* const* camera_ids,
                          const char* const* rig_camera_ids, int fixed);
/* AddRigInstancePositionPrior (bundle_adjuster.cc:200-217). */
int gbba_add_rig_instance_position_prior(gbba_adjuster_t* h, const char* id, const double* position,
                                         const double* std_dev, const char* scale_group);
/* AddPoint (bundle_adjuster.cc:246-258). */
int gbba_add_point(gbba_adjuster_t* h, const char* id, const double* position, int constant);
/* Absolute orientation constraints of a shot, each under CauchyLoss(1):
 * BundleAdjuster::AddAbsoluteUpVector / Pan / Tilt / Roll
 * (bundle_adjuster.cc:352-387, added to the problem at :1011-1082;
 * residuals absolute_motion_errors.h:10-126).  The up vector is a direction
 * in the camera frame that the shot rotation must take to world +z; the
 * angles in radians.  Constraints with std_deviation <= 0 are ignored, as
 * in the reference.  Evaluated on the host in FP64 (a few residuals per
 * shot); IRLS reweights them in the groups UP, PAN, TILT and ROLL.  An
 * unknown shot is GBBA_ERR_OUT_OF_RANGE here (the reference's shots_.at()
 * throws std::out_of_range when Run adds the block). */
int gbba_add_absolute_up_vector(gbba_adjuster_t* h, const char* shot_id, const double* up_vector,
                                double std_deviation);
int gbba_add_absolute_pan(gbba_adjuster_t* h, const char* shot_id, double angle, double std_deviation);
int gbba_add_absolute_tilt(gbba_adjuster_t* h, const char* shot_id, double angle, double std_deviation);
int gbba_add_absolute_roll(gbba_adjuster_t* h, const char* shot_id, double angle, double std_deviation);
/* The scaled residuals (before the loss) of one orientation constraint and
 * their Jacobian: the functors of absolute_motion_errors.h:10-126 at rig
 * instance rotation `instance_rotation` and rig camera rotation
 * `camera_rotation` (angle-axis; NULL: identity).  kind 0 up vector
 * (target[0..2]), 1 pan, 2 tilt, 3 roll (target[0]).  Writes m = 3 (up
 * vector) or 1 residuals and J[m][6] (d/d instance rotation, d/d rig camera
 * rotation), and m to *n_residuals.  Host arithmetic only. */
int gbba_orientation_residual(int kind, const double* target, double std_deviation,
                              const double* instance_rotation, const double* camera_rotation, double* residuals,
                              double* jacobian, int* n_residuals);
/* Constraints between shots, evaluated on the host in FP64 like the
 * orientation constraints.  Unknown shots are GBBA_ERR_OUT_OF_RANGE when the
 * constraint is added.
 *   AddRelativeRotation (bundle_adjuster.cc:307-309, added at :912-956):
 *     residual scale_matrix * log(R_ij R_i^T R_j) (RelativeRotationError,
 *     relative_motion_errors.h:66-94); scale_matrix row-major 3 x 3, NULL
 *     for the identity; under the relative-motion loss, IRLS group ROT.
 *   AddCommonPosition (bundle_adjuster.cc:311-320, :958-999): the two shot
 *     positions agree, horizontally within `margin`
 *     (CommonPositionError, relative_motion_errors.h:96-126); TukeyLoss(1),
 *     group POS.
 *   AddLinearMotion (bundle_adjuster.cc:503-514, :1080-1138): shot1 at
 *     fraction alpha between shot0 and shot2 in position and rotation
 *     (LinearMotionError, motion_prior_errors.h:12-74); CauchyLoss(1),
 *     group MOTION.
 * SetRelativeMotionLossFunction (bundle_adjuster.cc:396-400): the loss of
 * the relative rotations; an unknown name fails the run that needs it. */
int gbba_add_relative_rotation(gbba_adjuster_t* h, const char* shot_i, const char* shot_j, const double* rotation,
                               const double* scale_matrix);
int gbba_add_common_position(gbba_adjuster_t* h, const char* shot_i, const char* shot_j, double margin,
                             double std_deviation);
int gbba_add_linear_motion(gbba_adjuster_t* h, const char* shot0, const char* shot1, const char* shot2,
                           double alpha, double position_std_deviation, double orientation_std_deviation);
int gbba_set_relative_motion_loss_function(gbba_adjuster_t* h, const char* name, double threshold);
/* SetGaugeFixShots (bundle_adjuster.cc:389-394): the origin shot's rig
 * instance becomes constant and a run adds log(|t1 - t2| / d) on the two
 * shots' rig instance positions, d their distance when the run starts
 * (TranslationPriorError, absolute_motion_errors.h:175-190; added at
 * bundle_adjuster.cc:1140-1157), no loss, group GAUGE. */
int gbba_set_gauge_fix_shots(gbba_adjuster_t* h, const char* shot_origin, const char* shot_scale);
/* AddHeatmap (bundle_adjuster.cc:331-336): a cost grid of n values,
 * row-major with `width` columns (n a multiple of width), `resolution`
 * metres per cell; an id added again replaces its grid.
 * AddAbsolutePositionHeatmap (:338-350, added at :1000-1009): the grid's
 * bicubic (Catmull-Rom, border-clamped) value at the shot position,
 * row = height / 2 - (y - y_offset) / resolution, column = width / 2 +
 * (x - x_offset) / resolution, divided by std_deviation
 * (HeatmapdCostFunctor, absolute_motion_errors.h:128-173); no loss, group
 * HEATMAP.  Unknown shots or heatmap ids are GBBA_ERR_OUT_OF_RANGE. */
int gbba_add_heatmap(gbba_adjuster_t* h, const char* heatmap_id, const double* data, int64_t n, int64_t width,
                     double resolution);
int gbba_add_absolute_position_heatmap(gbba_adjuster_t* h, const char* shot_id, const char* heatmap_id,
                                       double x_offset, double y_offset, double std_deviation);
/* rho(s), rho'(s), rho''(s) of the host constraint losses: kind 0 trivial,
 * 1 Huber, 2 soft-L1, 3 Cauchy, 4 arctan (the names of
 * set_relative_motion_loss_function), 5 Tukey, at scale a.  Host arithmetic
 * only. */
int gbba_host_loss(int kind, double a, double s, double* rho);
/* The heatmap residual at instance pose [6] and rig camera pose [6] (NULL:
 * none) and its Jacobian [12] (instance rotation, instance position, rig
 * camera rotation, rig camera position).  Host arithmetic only. */
int gbba_heatmap_residual(const double* grid, int64_t n, int64_t width, double resolution, double x_offset,
                          double y_offset, double std_deviation, const double* instance_pose,
                          const double* rig_camera_pose, double* residual, double* jacobian);
/* Reconstructions (bundle_adjuster.cc:219-244): AddReconstruction,
 * AddReconstructionInstance (an unknown reconstruction id is ignored, as in
 * the reference), SetScaleSharing (one scale for the whole reconstruction:
 * its first instance's in id order), and Reconstruction::GetScale after a
 * run (the shared scale, or the instance's).  The scales are unknowns of the
 * relative motions only; the reference's lower bound 0 is not enforced. */
int gbba_add_reconstruction(gbba_adjuster_t* h, const char* id, int constant);
int gbba_add_reconstruction_instance(gbba_adjuster_t* h, const char* reconstruction_id, double scale,
                                     const char* instance_id);
int gbba_set_scale_sharing(gbba_adjuster_t* h, const char* id, int share);
int gbba_get_reconstruction_scale(const gbba_adjuster_t* h, const char* reconstruction_id, const char* instance_id,
                                  double* scale);
/* 1 when the reconstruction exists, else 0 (-1: invalid handle). */
int gbba_has_reconstruction(const gbba_adjuster_t* h, const char* reconstruction_id);
/* AddRelativeMotion (bundle_adjuster.cc:303-305, added at :872-910): the
 * motion [rx ry rz tx ty tz scale] from rig instance i to j with a 7 x 7
 * row-major scale matrix (NULL: identity), under the relative-motion loss
 * at threshold x robust_multiplier, IRLS group REL (RelativeMotionError,
 * relative_motion_errors.h:13-64).  Both instances must belong to a
 * reconstruction when the run starts (else GBBA_ERR_OUT_OF_RANGE). */
int gbba_add_relative_motion(gbba_adjuster_t* h, const char* instance_i, const char* instance_j,
                             const double* motion, double robust_multiplier, int observed_scale,
                             const double* scale_matrix);
/* SetAdjustAbsolutePositionStd (bundle_adjuster.cc:402-404, used at
 * :772-838): with adjust != 0 a run divides the GPS priors of each scale
 * group by a std multiplier it optimises (from 1), regularised by
 * log(1 / sqrt(2 pi m^2)) (StdDeviationConstraint); IRLS groups GPS and
 * STDDEV.  Batched solves reject it. */
int gbba_set_adjust_absolute_position_std(gbba_adjuster_t* h, int adjust);
/* The scaled residuals (before the loss) of one constraint between shots
 * and their Jacobian.  kind 0 relative rotation (params: rotation[3], then
 * the row-major scale matrix [9]), 1 common position (params: margin,
 * std_deviation), 2 linear motion (params: alpha, position std, orientation
 * std), 3 gauge scale (params: the distance; rig camera poses unused), 5
 * relative motion (params: motion[7], observed-scale flag, scale matrix
 * [49], scale_i, scale_j; rig camera poses unused; the scales' columns are
 * 24 and 25), 6 adjusted GPS prior (params: prior[3], std[3], multiplier;
 * one instance pose; the multiplier's column is 24), 7 std-multiplier
 * regulariser (params: multiplier; no pose; column 24), 8 the GPS prior of
 * kind 6 through an optimised camera bias (params: prior[3], std[3],
 * multiplier, bias rotation[3], translation[3], scale; the bias rotation
 * and translation's columns are 6..11, its scale's 25).
 * instance_poses[n][6] and rig_camera_poses[n][6] (NULL: no rig
 * cameras) for the n = 2 (3 for linear motion) shots, [rx ry rz tx ty tz]
 * with t the position.  Writes m = 3 (6 for linear motion, 1 for the gauge
 * scale and the regulariser, 7 for a relative motion) residuals, J[m][36]
 * (12 columns per shot: instance rotation, instance position, rig camera
 * rotation, rig camera position) and m to *n_residuals.  Host arithmetic
 * only. */
int gbba_relative_residual(int kind, const double* instance_poses, const double* rig_camera_poses,
                           const double* params, double* residuals, double* jacobian, int* n_residuals);
/* AddPointPrior (bundle_adjuster.cc:260-272). */
int gbba_add_point_prior(gbba_adjuster_t* h, const char* id, const double* position, const double* std_dev,
                         int has_altitude);
/* AddPointProjectionObservation (bundle_adjuster.cc:274-287). */
int gbba_add_point_projection_observation(gbba_adjuster_t* h, const char* shot, const char* point,
                                          const double* observation, double std_dev, int is_gcp);

/* Index-based bulk interface, the counterpart of GetShotRaw / GetPointRaw /
 * AddPointProjectionObservationRaw (bundle_adjuster.cc:289-301, 1336-1338,
 * 1377-1379) used by sfm::BAHelpers.  Indices are assigned in insertion
 * order; -1 when the id is unknown. */
int64_t gbba_shot_index(const gbba_adjuster_t* h, const char* shot);
int64_t gbba_point_index(const gbba_adjuster_t* h, const char* point);
/* Adds n points; ids may be NULL (ids are then the decimal point indices). */
int gbba_add_points_bulk(gbba_adjuster_t* h, int64_t n, const double* xyz, const uint8_t* constant,
                         const char* const* ids, int64_t* first_index);
int gbba_add_point_projection_observations_bulk(gbba_adjuster_t* h, int64_t n, const int32_t* shot_index,
                                                const int32_t* point_index, const double* xy,
                                                const double* std_dev, const uint8_t* is_gcp);
/* The depth_prior argument of AddPointProjectionObservation
 * (bundle_adjuster.cc:274-301, pybind.cc:94-100): map::Depth {value,
 * is_radial, std_deviation} (map/observation.h:10-18) attached to n
 * observations given by their insertion index (0-based, over every
 * observation added so far, string or bulk).  At Run each becomes a
 * RelativeDepthError residual (bundle_adjuster.cc:572-604,
 * bundle/error/relative_depth_error.h) in the IRLS group "DEPTH", under the
 * point-projection loss; value and std are stored as floats, as map::Depth
 * holds them.  is_radial may be NULL (radial).  A std that is not positive
 * is GBBA_ERR_INVALID_ARGUMENT; a non-finite value fails at gbba_run with
 * GBBA_ERR_RUNTIME ("<shot> has non-finite depth prior", :582-586). */
int gbba_set_observation_depth_priors(gbba_adjuster_t* h, int64_t n, const int64_t* observation_index,
                                      const double* value, const double* std_dev, const uint8_t* is_radial);

/* Settings (bundle_adjuster.cc:400-483).  The point-projection loss
 * (pybundle.pyi:131) takes the names of CreateLossFunction
 * (bundle_adjuster.cc:485-499). */
int gbba_set_point_projection_loss_function(gbba_adjuster_t* h, const char* name, double threshold);
/* IRLS reweighting of projection residuals: 1 mixture (the reference's
 * behaviour, default), 0 none (fixed objective with the robust loss). */
int gbba_set_irls_mode(gbba_adjuster_t* h, int mode);
/* GBBA_PRECISION_MIXED (default) or GBBA_PRECISION_FP64. */
int gbba_set_precision(gbba_adjuster_t* h, int precision);
int gbba_set_max_num_iterations(gbba_adjuster_t* h, int n);
int gbba_set_num_threads(gbba_adjuster_t* h, int n);
int gbba_set_use_analytic_derivatives(gbba_adjuster_t* h, int use);
int gbba_set_linear_solver_type(gbba_adjuster_t* h, const char* type);
int gbba_set_internal_parameters_prior_sd(gbba_adjuster_t* h, double focal_sd, double aspect_ratio_sd, double c_sd,
                                          double k1_sd, double k2_sd, double p1_sd, double p2_sd, double k3_sd,
                                          double k4_sd);
int gbba_set_rig_parameters_prior_sd(gbba_adjuster_t* h, double translation_sd, double rotation_sd);
int gbba_set_compute_reprojection_errors(gbba_adjuster_t* h, int v);
int gbba_set_compute_covariances(gbba_adjuster_t* h, int v);
int gbba_get_covariance_estimation_valid(const gbba_adjuster_t* h);
/* The 6 x 6 row-major covariance of a rig instance's pose [rx ry rz tx ty tz]
 * after a run with covariances on, as BundleAdjuster::ComputeCovariances
 * stores it in the rig instance (bundle_adjuster.cc:1217-1287): the instance
 * block of the inverse Gauss-Newton matrix at the final state (locked
 * coordinates zero), computed when the reduced camera system has at most
 * 4,096 optimised unknowns; otherwise, or if it is singular, the estimation
 * is invalid and the reference's default (variances 1e-5 rotation, 1e-2
 * translation) is stored. */
int gbba_get_rig_instance_covariance(const gbba_adjuster_t* h, const char* id, double* out);
int gbba_set_skip_initial_reweighting(gbba_adjuster_t* h, int v);
int gbba_set_default_density_ratio(gbba_adjuster_t* h, double ratio);
double gbba_get_default_density_ratio(const gbba_adjuster_t* h);
int gbba_set_group_density_ratio(gbba_adjuster_t* h, const char* group, double ratio);
double gbba_get_group_density_ratio(const gbba_adjuster_t* h, const char* group);
/* Relative residual at which the reduced-camera-system PCG stops. */
int gbba_set_pcg_tolerance(gbba_adjuster_t* h, double tolerance);
/* Jacobian storage of the iterative solver.  0 (default): the residual +
 * Jacobian records of a linearization are stored (two copies, about 224 B
 * per observation for a perspective camera in mixed precision) when they
 * fit in device memory, and otherwise evaluated again in every pass
 * (matrix-free); 1: always matrix-free; -1: always stored.  The exact dense
 * path always stores them. */
int gbba_set_matrix_free(gbba_adjuster_t* h, int mode);
/* How the PCG iterations are launched.  1 (default): all of a linear
 * solve's iterations as one CUDA graph launch, with the stopping test on the
 * device; 0: kernel by kernel with the scalars read on the host every
 * iteration (the same kernels and results; a profiler sees each launch --
 * kernels inside a graph with a conditional node are not profiled one by
 * one).  Sharded solves always launch kernel by kernel. */
int gbba_set_pcg_graph(gbba_adjuster_t* h, int enable);
/* Two-level PCG preconditioner for large blocks (an extension: Ceres'
 * ITERATIVE_SCHUR, bundle_adjuster.cc:1159-1190, preconditions with the
 * Schur-Jacobi blocks only).  leaf > 0 adds a coarse space: the rig
 * instances are split into spatial clusters of at most `leaf` instances
 * (more when the coarse system would pass 4096 unknowns), each with its
 * seven similarity modes; the coarse matrix is probed with 7 Schur products
 * per colour of a distance-2 colouring of the clusters once per
 * linearization.  0 (default): block-Jacobi only.  PCG solves only (not the
 * exact dense path, not sharded solves). */
int gbba_set_coarse_preconditioner(gbba_adjuster_t* h, int leaf);
/* The coarse space of the last run: clusters, colours, and the Schur
 * products spent probing the coarse matrix (all 0 when it was not used). */
int gbba_get_coarse_info(const gbba_adjuster_t* h, int* clusters, int* colours, int64_t* probes);
/* The coarse space the current problem would get (host only, no solve):
 * the cluster of every rig instance in insertion order (-1: no free
 * coordinate; cluster_of_instance holds n_instances entries), the colour of
 * every cluster (colour_of_cluster holds up to cluster_capacity entries),
 * and the counts. */
int gbba_coarse_space_layout(gbba_adjuster_t* h, int leaf, int* cluster_of_instance, int64_t n_instances,
                             int* colour_of_cluster, int cluster_capacity, int* clusters, int* colours);

/* ---- Point-partitioned (sharded) solve over several GPUs
 *
 * No counterpart in the reference, which scales out by rounds of local
 * bundles (sfm::BAHelpers::BundleStochastic, ba_helpers.cc:1231-1370).
 * One adjuster per rank (one process or thread per GPU), each given the
 * whole problem.  A rank solves with the points gbba_get_shard_points
 * assigns it and all of their observations; cameras, rig cameras and rig
 * instances are held by every rank.  The ranks exchange, through the
 * caller's all-reduce: the camera-side gradient and column norms of each
 * linearization, the Schur right-hand side and preconditioner blocks of
 * each step, the Schur product of each PCG iteration (one camera-sized
 * vector), rank 0's PCG scalars and camera step, and the scalar sums (cost,
 * model decrease, step norm, IRLS group statistics).  The steps come from
 * PCG (the dense path and the covariances are single-rank).  After gbba_run
 * every rank holds the same camera side and the solved values of its own
 * points; another rank's points keep their values from before the run, and
 * their reprojection errors and weights read back as NaN.
 *
 * allreduce(ctx, data, count, op) reduces `count` doubles in host memory in
 * place over the ranks (op GBBA_REDUCE_SUM or GBBA_REDUCE_MAX) and returns
 * 0, or nonzero on failure (gbba_run then fails with GBBA_ERR_RUNTIME).
 * Every rank makes the same sequence of calls.  world_size 1 (the default)
 * is the ordinary single-GPU solve. */
#define GBBA_REDUCE_SUM 0
#define GBBA_REDUCE_MAX 1
typedef int (*gbba_allreduce_fn)(void* ctx, double* data, int64_t count, int op);
int gbba_set_shard(gbba_adjuster_t* h, int rank, int world_size, gbba_allreduce_fn allreduce, void* ctx);
/* Points [*first, *last) (insertion order) that `rank` solves with under
 * the adjuster's world size: contiguous ranges with nearly equal numbers of
 * observations. */
int gbba_get_shard_points(const gbba_adjuster_t* h, int rank, int64_t* first, int64_t* last);

/* BundleAdjuster::Run (bundle_adjuster.cc:670-1203). */
int gbba_run(gbba_adjuster_t* h);

/* Getters (bundle_adjuster.cc:1303-1399). */
int gbba_get_camera(const gbba_adjuster_t* h, const char* id, int* projection, double* values, int capacity,
                    int* n_values);
int gbba_get_rig_instance_pose(const gbba_adjuster_t* h, const char* id, double* pose);
int gbba_get_rig_camera_pose(const gbba_adjuster_t* h, const char* id, double* pose);
int gbba_get_point(const gbba_adjuster_t* h, const char* id, double* position);
int gbba_has_point(const gbba_adjuster_t* h, const char* id);
int64_t gbba_num_projections(const gbba_adjuster_t* h);
int64_t gbba_num_points(const gbba_adjuster_t* h);
int gbba_get_points_bulk(const gbba_adjuster_t* h, int64_t first, int64_t n, double* xyz);
/* Per observation (insertion order): unscaled residual (std = 1) padded to
 * 3 values, IRLS weight, residual dimension (ComputeReprojectionErrors and
 * RetrieveProjectionWeights, bundle_adjuster.cc:1205-1216, 1289-1301). */
int gbba_get_projection_results(const gbba_adjuster_t* h, int64_t n, double* errors, double* weights,
                                int32_t* dims);
/* Reports; return the full length of the text (written up to len - 1
 * bytes, NUL-terminated), -1 on error. */
int gbba_brief_report(const gbba_adjuster_t* h, char* buf, size_t len);
int gbba_full_report(const gbba_adjuster_t* h, char* buf, size_t len);
int gbba_irls_report(const gbba_adjuster_t* h, char* buf, size_t len);

typedef struct gbba_summary {
  double initial_cost;
  double final_cost;
  double seconds;
  double linear_solver_seconds;
  double jacobian_seconds;
  double residual_seconds;
  int iterations;
  int successful_steps;
  int unsuccessful_steps;
  int usable;
  int64_t kernel_launches;
  double setup_seconds; /* problem setup inside run(): sorts, uploads */
  int64_t linear_solver_failures; /* dense factorizations of a damped system that was not positive definite */
} gbba_summary_t;
int gbba_get_summary(const gbba_adjuster_t* h, gbba_summary_t* out);
/* Iteration trace of the last run: records of 8 doubles
 * [iteration, cost, seconds since start, success, linear iterations,
 *  trust-region radius, relative decrease, step norm]. */
int gbba_get_trace(const gbba_adjuster_t* h, int capacity, double* records, int* n);

/* ------------------------------------------------------------------------
 * Batched runs: many adjusters solved together on the GPU.  The reference
 * runs one bundle::BundleAdjuster per local bundle adjustment
 * (sfm::BAHelpers::BundleLocal, ba_helpers.cc:442-804); a batch solves many
 * such problems in one device layout, with per-problem trust regions and
 * PCG scalars on the device and one LM iteration recorded as a CUDA graph.
 * Each adjuster is filled as usual; after gbba_batch_run its getters and
 * reports hold its own result.  Batches take fixed intrinsics and rig
 * cameras and no priors (as BundleLocal, ba_helpers.cc:478-486); IRLS is
 * not applied; every adjuster needs the same loss function.  The adjusters
 * are borrowed and must outlive the batch's use of them. */
typedef struct gbba_batch gbba_batch_t;
gbba_batch_t* gbba_batch_create(void);
void gbba_batch_destroy(gbba_batch_t* b);
int gbba_batch_add(gbba_batch_t* b, gbba_adjuster_t* h);
int gbba_batch_size(const gbba_batch_t* b);
/* precision GBBA_PRECISION_*; LM iterations; PCG iterations per LM step;
 * PCG relative tolerance; use_graph 2 (default in the bindings): the whole
 * LM loop as one CUDA graph launch, a device-side while node that ends when
 * every problem is done or max_iterations are taken; 1: one recorded LM
 * iteration replayed per iteration with a host check between them; 0:
 * kernel by kernel; pick the slot-kernel grid by timing (1). */
int gbba_batch_set_options(gbba_batch_t* b, int precision, int max_iterations, int pcg_iterations,
                           double pcg_tolerance, int use_graph, int autotune);
/* The linear solver type of the batch's steps, as
 * BundleAdjuster::SetLinearSolverType (bundle_adjuster.cc:482) names them
 * and sfm::BAHelpers picks them for local bundles (DENSE_SCHUR,
 * ba_helpers.cc:336-337).  An exact type (DENSE_SCHUR, DENSE_QR,
 * DENSE_NORMAL_CHOLESKY, SPARSE_SCHUR, SPARSE_NORMAL_CHOLESKY) makes every
 * step exact: FP64 records whatever precision was set, and PCG to a 1e-10
 * relative residual with at least as many iterations as the largest
 * problem has camera-side unknowns.  ITERATIVE_SCHUR or CGNR (the default):
 * the options' precision and PCG.  Unknown names: GBBA_ERR_INVALID_ARGUMENT. */
int gbba_batch_set_linear_solver(gbba_batch_t* b, const char* type);
/* A problem has converged when an accepted step changes its cost by at
 * most tolerance * cost (default 1e-7, as gbba_run's convergence test). */
int gbba_batch_set_function_tolerance(gbba_batch_t* b, double tolerance);
int gbba_batch_run(gbba_batch_t* b);
typedef struct gbba_batch_summary {
  double seconds;        /* whole run, set-up included */
  double setup_seconds;  /* layout, uploads, first linearization, autotuning */
  double solve_seconds;  /* the LM iterations */
  int lm_iterations;     /* iterations of the batch (its slowest problem) */
  int grid;              /* slot-kernel grid the autotuner chose */
  int n_problems;
  int n_converged;
  int64_t graph_nodes;   /* nodes of the recorded LM iteration */
  int64_t kernel_launches;
  int64_t graph_launches;  /* graph launches of the LM loop: 1 with the device-side loop */
} gbba_batch_summary_t;
int gbba_batch_get_summary(const gbba_batch_t* b, gbba_batch_summary_t* out);

/* ---- Post-solve outlier selection
 *
 * The observation test of sfm::BAHelpers::RemoveOutliers
 * (ba_helpers.cc:1847-1975), data-parallel on the device.  filter_type 0
 * (FIXED) uses fixed_threshold; 1 (AUTO) computes it from all observations'
 * 2D errors: componentwise medians m (the element of rank n/2), robust
 * deviation s = 1.486 * median |e - m|, threshold = auto_ratio *
 * |(m_x + s, m_y + s)|.  An observation is an outlier if |e|^2 >
 * threshold^2 or its IRLS weight is below weight_threshold.  A point is
 * removed if it loses an observation and keeps fewer than two.  Defaults
 * of the reference's configuration: FIXED, 0.006, 3.0, 0.5. */
typedef struct gbba_outlier_config {
  int filter_type;
  double fixed_threshold;
  double auto_ratio;
  double weight_threshold;
} gbba_outlier_config_t;
typedef struct gbba_outlier_result {
  double threshold;
  int64_t n_outliers;
  int64_t n_removed_points;
  double device_seconds; /* stream time from the inputs resident to the flags written (host scans included) */
} gbba_outlier_result_t;
/* errors: n rows of `stride` doubles (columns 0 and 1 are the 2D error),
 * weights [n], obs_point [n] in [0, n_points); host buffers.  flags [n]
 * (1: outlier) and point_removed [n_points] are written. */
int gbba_find_outliers(const double* errors, int stride, const double* weights, const int32_t* obs_point, int64_t n,
                       int64_t n_points, const gbba_outlier_config_t* config, uint8_t* flags, uint8_t* point_removed,
                       gbba_outlier_result_t* result);
/* The same on an adjuster's last solve (its reprojection errors and IRLS
 * weights, observations and points in insertion order). */
int gbba_adjuster_find_outliers(const gbba_adjuster_t* h, const gbba_outlier_config_t* config, uint8_t* flags,
                                uint8_t* point_removed, gbba_outlier_result_t* result);

/* ---- Dense reduced-camera-system solver
 *
 * The linear solver behind gbba_run's dense mode (linear solver types
 * DENSE_SCHUR, DENSE_QR and DENSE_NORMAL_CHOLESKY, and SPARSE_SCHUR /
 * SPARSE_NORMAL_CHOLESKY up to a few thousand camera-side unknowns): the
 * GPU counterpart of the Cholesky factorization Ceres' DENSE_SCHUR and
 * SPARSE_SCHUR solvers apply to the reduced camera system
 * (bundle_adjuster.cc:1159-1190; DENSE_SCHUR up to 200 shots in
 * sfm::BAHelpers, ba_helpers.cc:42-49).  Exposed on its own for callers
 * that form such systems themselves, and for tests.
 *
 * gbba_dense_spd_solve solves A x = b for a symmetric positive definite
 * n x n row-major FP64 matrix (host buffers; the lower triangle is read).
 * The factorization runs on the tensor cores (TF32 operands, three products
 * per term for FP32 accuracy) after a symmetric Jacobi scaling; conjugate
 * gradients in FP64 on the FP64 matrix, preconditioned by that factor, then
 * drive the scaled residual |D (b - A x)| / |D b| below tol, D =
 * diag(A)^-1/2, within max_refinements
 * iterations (one FP64 matrix-vector product each).  status: 0 solved, 1
 * not positive definite, 2 a device wait timed out, 3 not converged to tol
 * within max_refinements iterations (x is the last iterate). */
typedef struct gbba_dense_stats {
  int status;
  int refinements;
  double rel_residual;
  double factor_seconds;
  double solve_seconds;
} gbba_dense_stats_t;
int gbba_dense_spd_solve(const double* a, int n, const double* b, double* x, double tol, int max_refinements,
                         gbba_dense_stats_t* stats);
/* C = A B^T on the tensor cores for row-major FP32 A (m x k), B (n x k),
 * C (m x n), host buffers; m and n multiples of 128, k a multiple of 32.
 * The product kernel of the factorization, exposed for tests. */
int gbba_dense_gemm_nt(const float* a, const float* b, float* c, int m, int n, int k);

#ifdef __cplusplus
}
#endif

#endif /* GBBA_H_ */
