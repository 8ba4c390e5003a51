"""Drop-in for ``opensfm.pybundle`` (bundle adjustment on the GPU).

``BundleAdjuster`` has the method names, argument order and error behaviour
of the reference's pybind module (opensfm/src/lib/bundle/python/pybind.cc:
60-147, pybundle.pyi:31-134) and forwards every call to the C ABI of
libgbba.so (include/gbba.h).  Unknown ids raise ``RuntimeError``, an unknown
shot or point in ``add_point_projection_observation`` raises ``IndexError``
(std::out_of_range in the reference).

Beyond the reference's methods it exposes bulk (numpy) adders for large
problems, the precision / IRLS switches of the GPU solver and the iteration
trace.  The one feature that the GPU solver does not implement (optimised
camera biases) raises ``NotImplementedError`` instead of being silently
ignored.
"""
from __future__ import annotations

import ctypes as C
from typing import Dict, Optional

import numpy as np

from . import _lib
from .pygeometry import Camera, Pose, Similarity

_D = C.POINTER(C.c_double)
_I32 = C.POINTER(C.c_int32)
_U8 = C.POINTER(C.c_uint8)
_H = C.c_void_p
# int allreduce(void* ctx, double* data, int64_t count, int op)
ALLREDUCE_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.POINTER(C.c_double), C.c_int64, C.c_int)


class Summary(C.Structure):
    _fields_ = [("initial_cost", C.c_double), ("final_cost", C.c_double), ("seconds", C.c_double),
                ("linear_solver_seconds", C.c_double), ("jacobian_seconds", C.c_double),
                ("residual_seconds", C.c_double), ("iterations", C.c_int), ("successful_steps", C.c_int),
                ("unsuccessful_steps", C.c_int), ("usable", C.c_int), ("kernel_launches", C.c_int64),
                ("setup_seconds", C.c_double), ("linear_solver_failures", C.c_int64)]


def _declare(L) -> None:
    if getattr(L, "_gbba_adjuster_declared", False):
        return
    S = C.c_char_p
    sig = {
        "gbba_create": ([], _H),
        "gbba_destroy": ([_H], None),
        "gbba_add_camera": ([_H, S, C.c_int, _D, _D, C.c_int, C.c_int], C.c_int),
        "gbba_set_camera_bias": ([_H, S, _D, _D, C.c_double], C.c_int),
        "gbba_set_camera_bias_parameters": ([_H, S, _I32, C.c_int], C.c_int),
        "gbba_get_bias": ([_H, S, _D, _D, C.POINTER(C.c_double)], C.c_int),
        "gbba_add_rig_camera": ([_H, S, _D, _D, C.c_int], C.c_int),
        "gbba_add_rig_instance": ([_H, S, _D, C.c_int, C.POINTER(S), C.POINTER(S), C.POINTER(S), C.c_int], C.c_int),
        "gbba_add_rig_instance_position_prior": ([_H, S, _D, _D, S], C.c_int),
        "gbba_add_point": ([_H, S, _D, C.c_int], C.c_int),
        "gbba_add_point_prior": ([_H, S, _D, _D, C.c_int], C.c_int),
        "gbba_add_absolute_up_vector": ([_H, S, _D, C.c_double], C.c_int),
        "gbba_add_absolute_pan": ([_H, S, C.c_double, C.c_double], C.c_int),
        "gbba_add_absolute_tilt": ([_H, S, C.c_double, C.c_double], C.c_int),
        "gbba_add_absolute_roll": ([_H, S, C.c_double, C.c_double], C.c_int),
        "gbba_orientation_residual": ([C.c_int, _D, C.c_double, _D, _D, _D, _D, C.POINTER(C.c_int)], C.c_int),
        "gbba_add_relative_rotation": ([_H, S, S, _D, _D], C.c_int),
        "gbba_add_common_position": ([_H, S, S, C.c_double, C.c_double], C.c_int),
        "gbba_add_linear_motion": ([_H, S, S, S, C.c_double, C.c_double, C.c_double], C.c_int),
        "gbba_set_relative_motion_loss_function": ([_H, S, C.c_double], C.c_int),
        "gbba_relative_residual": ([C.c_int, _D, _D, _D, _D, _D, C.POINTER(C.c_int)], C.c_int),
        "gbba_set_gauge_fix_shots": ([_H, S, S], C.c_int),
        "gbba_add_reconstruction": ([_H, S, C.c_int], C.c_int),
        "gbba_add_reconstruction_instance": ([_H, S, C.c_double, S], C.c_int),
        "gbba_set_scale_sharing": ([_H, S, C.c_int], C.c_int),
        "gbba_get_reconstruction_scale": ([_H, S, S, _D], C.c_int),
        "gbba_has_reconstruction": ([_H, S], C.c_int),
        "gbba_set_adjust_absolute_position_std": ([_H, C.c_int], C.c_int),
        "gbba_add_relative_motion": ([_H, S, S, _D, C.c_double, C.c_int, _D], C.c_int),
        "gbba_add_heatmap": ([_H, S, _D, C.c_int64, C.c_int64, C.c_double], C.c_int),
        "gbba_add_absolute_position_heatmap": ([_H, S, S, C.c_double, C.c_double, C.c_double], C.c_int),
        "gbba_heatmap_residual": ([_D, C.c_int64, C.c_int64, C.c_double, C.c_double, C.c_double, C.c_double, _D, _D,
                                   _D, _D], C.c_int),
        "gbba_add_point_projection_observation": ([_H, S, S, _D, C.c_double, C.c_int], C.c_int),
        "gbba_shot_index": ([_H, S], C.c_int64),
        "gbba_point_index": ([_H, S], C.c_int64),
        "gbba_add_points_bulk": ([_H, C.c_int64, _D, _U8, C.POINTER(S), C.POINTER(C.c_int64)], C.c_int),
        "gbba_add_point_projection_observations_bulk": ([_H, C.c_int64, _I32, _I32, _D, _D, _U8], C.c_int),
        "gbba_set_point_projection_loss_function": ([_H, S, C.c_double], C.c_int),
        "gbba_set_irls_mode": ([_H, C.c_int], C.c_int),
        "gbba_set_precision": ([_H, C.c_int], C.c_int),
        "gbba_set_max_num_iterations": ([_H, C.c_int], C.c_int),
        "gbba_set_num_threads": ([_H, C.c_int], C.c_int),
        "gbba_set_use_analytic_derivatives": ([_H, C.c_int], C.c_int),
        "gbba_set_linear_solver_type": ([_H, S], C.c_int),
        "gbba_set_internal_parameters_prior_sd": ([_H] + [C.c_double] * 9, C.c_int),
        "gbba_set_rig_parameters_prior_sd": ([_H, C.c_double, C.c_double], C.c_int),
        "gbba_set_compute_reprojection_errors": ([_H, C.c_int], C.c_int),
        "gbba_set_compute_covariances": ([_H, C.c_int], C.c_int),
        "gbba_get_covariance_estimation_valid": ([_H], C.c_int),
        "gbba_get_rig_instance_covariance": ([_H, S, _D], C.c_int),
        "gbba_set_skip_initial_reweighting": ([_H, C.c_int], C.c_int),
        "gbba_set_default_density_ratio": ([_H, C.c_double], C.c_int),
        "gbba_get_default_density_ratio": ([_H], C.c_double),
        "gbba_set_group_density_ratio": ([_H, S, C.c_double], C.c_int),
        "gbba_get_group_density_ratio": ([_H, S], C.c_double),
        "gbba_set_pcg_tolerance": ([_H, C.c_double], C.c_int),
        "gbba_set_matrix_free": ([_H, C.c_int], C.c_int),
        "gbba_set_pcg_graph": ([_H, C.c_int], C.c_int),
        "gbba_set_coarse_preconditioner": ([_H, C.c_int], C.c_int),
        "gbba_get_coarse_info": ([_H, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int64)], C.c_int),
        "gbba_coarse_space_layout": ([_H, C.c_int, C.POINTER(C.c_int), C.c_int64, C.POINTER(C.c_int), C.c_int,
                                      C.POINTER(C.c_int), C.POINTER(C.c_int)], C.c_int),
        "gbba_set_shard": ([_H, C.c_int, C.c_int, ALLREDUCE_FN, C.c_void_p], C.c_int),
        "gbba_get_shard_points": ([_H, C.c_int, C.POINTER(C.c_int64), C.POINTER(C.c_int64)], C.c_int),
        "gbba_run": ([_H], C.c_int),
        "gbba_get_camera": ([_H, S, C.POINTER(C.c_int), _D, C.c_int, C.POINTER(C.c_int)], C.c_int),
        "gbba_get_rig_instance_pose": ([_H, S, _D], C.c_int),
        "gbba_get_rig_camera_pose": ([_H, S, _D], C.c_int),
        "gbba_get_point": ([_H, S, _D], C.c_int),
        "gbba_has_point": ([_H, S], C.c_int),
        "gbba_num_projections": ([_H], C.c_int64),
        "gbba_num_points": ([_H], C.c_int64),
        "gbba_set_observation_depth_priors": ([_H, C.c_int64, C.POINTER(C.c_int64), _D, _D, _U8], C.c_int),
        "gbba_get_points_bulk": ([_H, C.c_int64, C.c_int64, _D], C.c_int),
        "gbba_get_projection_results": ([_H, C.c_int64, _D, _D, _I32], C.c_int),
        "gbba_brief_report": ([_H, C.c_char_p, C.c_size_t], C.c_int),
        "gbba_full_report": ([_H, C.c_char_p, C.c_size_t], C.c_int),
        "gbba_irls_report": ([_H, C.c_char_p, C.c_size_t], C.c_int),
        "gbba_get_summary": ([_H, C.POINTER(Summary)], C.c_int),
        "gbba_get_trace": ([_H, C.c_int, _D, C.POINTER(C.c_int)], C.c_int),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    L._gbba_adjuster_declared = True


REDUCE_SUM = 0
REDUCE_MAX = 1


def torch_allreduce(group=None):
    """An all-reduce for BundleAdjuster.set_shard over a torch.distributed
    process group: gloo reduces the host array directly; NCCL through a copy
    on the current CUDA device."""
    import torch
    import torch.distributed as dist
    nccl = dist.get_backend(group) == "nccl"

    def f(a: np.ndarray, op: int) -> None:
        t = torch.from_numpy(a)
        rop = dist.ReduceOp.SUM if op == REDUCE_SUM else dist.ReduceOp.MAX
        if nccl:
            d = t.to("cuda")
            dist.all_reduce(d, op=rop, group=group)
            t.copy_(d.cpu())
        else:
            dist.all_reduce(t, op=rop, group=group)
    return f


def _b(s) -> bytes:
    if isinstance(s, bytes):
        return s
    return str(s).encode("utf-8")


def _vec(x, n: int) -> np.ndarray:
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float64).reshape(-1))
    if a.size != n:
        raise ValueError(f"expected {n} values, got {a.size}")
    return a


def _dp(a: np.ndarray):
    return a.ctypes.data_as(_D)


class RelativeMotion:
    """bundle::RelativeMotion (bundle_adjuster.h:75-104): the motion from
    rig instance i to j -- rotation, translation, scale -- its robust
    multiplier and whether the scale is observed; a 7 x 7 scale matrix."""

    def __init__(self, rig_instance_i: str, rig_instance_j: str, rotation, translation, scale: float,
                 robust_multiplier: float, observed_scale: bool) -> None:
        self.rig_instance_i = rig_instance_i
        self.rig_instance_j = rig_instance_j
        self.rotation = np.asarray(rotation, dtype=np.float64).reshape(3).copy()
        self.translation = np.asarray(translation, dtype=np.float64).reshape(3).copy()
        self.scale = float(scale)
        self.robust_multiplier = float(robust_multiplier)
        self.observed_scale = bool(observed_scale)
        self.scale_matrix = np.eye(7)

    def set_scale_matrix(self, s) -> None:
        self.scale_matrix = np.asarray(s, dtype=np.float64).reshape(7, 7).copy()


class Reconstruction:
    """bundle::Reconstruction as get_reconstruction returns it: get_scale
    reads the adjuster's current scale of an instance (the shared one when
    the reconstruction shares its scale)."""

    def __init__(self, ba: "BundleAdjuster", reconstruction_id: str) -> None:
        self._ba = ba
        self.id = reconstruction_id

    def get_scale(self, instance_id: str) -> float:
        v = C.c_double(0.0)
        self._ba._check(self._ba._L.gbba_get_reconstruction_scale(self._ba._h, _b(self.id), _b(instance_id),
                                                                   C.byref(v)))
        return v.value


class RelativeRotation:
    """bundle::RelativeRotation (bundle_adjuster.h:106-122): the rotation
    R_ij between shots i and j (angle-axis) and a 3 x 3 scale matrix."""

    def __init__(self, shot_i: str, shot_j: str, r) -> None:
        self.shot_i = shot_i
        self.shot_j = shot_j
        self.r = np.asarray(r, dtype=np.float64).reshape(3).copy()
        self.scale_matrix = np.eye(3)

    def set_scale_matrix(self, s) -> None:
        self.scale_matrix = np.asarray(s, dtype=np.float64).reshape(3, 3).copy()


class Point:
    """Result view of a point (bundle::Point, python/pybind.cc:51-58)."""

    def __init__(self, id: str, p: np.ndarray):
        self.id = id
        self.p = p
        self.reprojection_errors: Dict[str, np.ndarray] = {}
        self.reprojection_weights: Dict[str, float] = {}


class Depth:
    """map::Depth (opensfm/src/lib/map/observation.h:10-18, bound as
    ``pymap.Depth``): a depth prior of an observation.  value and
    std_deviation are floats (float32) in the reference; the adjuster
    rounds them the same way."""

    def __init__(self, value: float = 0.0, is_radial: bool = True, std_deviation: float = 1.0) -> None:
        self.value = value
        self.is_radial = is_radial
        self.std_deviation = std_deviation


class BundleAdjuster:
    """GPU bundle adjuster with the reference's pybind surface."""

    def __init__(self) -> None:
        self._L = _lib.lib()
        _declare(self._L)
        self._h = self._L.gbba_create()
        if not self._h:
            raise RuntimeError(self._L.gbba_last_error().decode())
        self._obs_keys: list = []      # (shot id, point id) per observation, when known
        self._shot_ids: list = []      # index -> id
        self._point_ids: Optional[list] = []

    def __del__(self) -> None:
        h = getattr(self, "_h", None)
        if h:
            self._L.gbba_destroy(h)
            self._h = None

    def _check(self, status: int) -> None:
        _lib.check(status)

    # -- cameras / rigs / points ------------------------------------------
    def add_camera(self, id: str, camera: Camera, prior: Camera, constant: bool) -> None:
        v = np.ascontiguousarray(camera.get_parameters_values(), np.float64)
        p = np.ascontiguousarray(prior.get_parameters_values(), np.float64)
        self._check(self._L.gbba_add_camera(self._h, _b(id), camera.model, _dp(v), _dp(p), v.size, int(constant)))

    def get_camera(self, id: str) -> Camera:
        vals = np.zeros(16)
        model = C.c_int(0)
        n = C.c_int(0)
        self._check(self._L.gbba_get_camera(self._h, _b(id), C.byref(model), _dp(vals), 16, C.byref(n)))
        cam = Camera(model.value, vals[: n.value])
        cam.id = id if isinstance(id, str) else id.decode()
        return cam

    def set_camera_bias(self, id: str, bias, parameters_to_optimize=()) -> None:
        """SetCameraBias (bundle_adjuster.cc:131-140): the bias (a
        ``pygeometry.Similarity``, or any object with rotation, translation
        and scale) and the indices of the parameters the run optimises
        (0-2 rotation, 3-5 translation, 6 scale)."""
        r = _vec(bias.rotation, 3)
        t = _vec(bias.translation, 3)
        self._check(self._L.gbba_set_camera_bias(self._h, _b(id), _dp(r), _dp(t), float(bias.scale)))
        idx = np.ascontiguousarray([int(i) for i in parameters_to_optimize], np.int32)
        self._check(self._L.gbba_set_camera_bias_parameters(self._h, _b(id), idx.ctypes.data_as(_I32), len(idx)))

    def get_bias(self, id: str) -> Similarity:
        r, t, s = np.zeros(3), np.zeros(3), C.c_double(1.0)
        self._check(self._L.gbba_get_bias(self._h, _b(id), _dp(r), _dp(t), C.byref(s)))
        return Similarity(r, t, s.value)

    def add_rig_camera(self, id: str, pose: Pose, pose_prior: Pose, fixed: bool) -> None:
        a = np.ascontiguousarray(pose.ba_data())
        b = np.ascontiguousarray(pose_prior.ba_data())
        self._check(self._L.gbba_add_rig_camera(self._h, _b(id), _dp(a), _dp(b), int(fixed)))

    def get_rig_camera_pose(self, id: str) -> Pose:
        d = np.zeros(6)
        self._check(self._L.gbba_get_rig_camera_pose(self._h, _b(id), _dp(d)))
        return Pose.from_ba_data(d)

    def add_rig_instance(self, id: str, pose: Pose, shot_cameras: Dict[str, str],
                         shot_rig_cameras: Dict[str, str], fixed: bool) -> None:
        shots = list(shot_cameras.keys())
        missing = [s for s in shots if s not in shot_rig_cameras]
        if missing:
            raise IndexError(f"unordered_map::at: shot {missing[0]} has no rig camera")
        n = len(shots)
        arr = C.c_char_p * max(n, 1)
        s_arr = arr(*[_b(s) for s in shots])
        c_arr = arr(*[_b(shot_cameras[s]) for s in shots])
        r_arr = arr(*[_b(shot_rig_cameras[s]) for s in shots])
        d = np.ascontiguousarray(pose.ba_data())
        self._check(self._L.gbba_add_rig_instance(self._h, _b(id), _dp(d), n, s_arr, c_arr, r_arr, int(fixed)))
        for s in shots:
            if s not in self._shot_ids:
                self._shot_ids.append(s)

    def get_rig_instance_pose(self, id: str) -> Pose:
        d = np.zeros(6)
        self._check(self._L.gbba_get_rig_instance_pose(self._h, _b(id), _dp(d)))
        return Pose.from_ba_data(d)

    def add_rig_instance_position_prior(self, id: str, position, std_deviation, scale_group: str) -> None:
        p = _vec(position, 3)
        s = _vec(std_deviation, 3)
        self._check(self._L.gbba_add_rig_instance_position_prior(self._h, _b(id), _dp(p), _dp(s), _b(scale_group)))

    def add_point(self, id: str, position, constant: bool) -> None:
        p = _vec(position, 3)
        self._check(self._L.gbba_add_point(self._h, _b(id), _dp(p), int(constant)))
        if self._point_ids is not None:
            self._point_ids.append(id)

    def add_point_prior(self, id: str, position, std_deviation, has_altitude: bool) -> None:
        p = _vec(position, 3)
        s = _vec(std_deviation, 3)
        self._check(self._L.gbba_add_point_prior(self._h, _b(id), _dp(p), _dp(s), int(has_altitude)))

    def has_point(self, id: str) -> bool:
        return bool(self._L.gbba_has_point(self._h, _b(id)))

    def get_point(self, id: str) -> Point:
        d = np.zeros(3)
        self._check(self._L.gbba_get_point(self._h, _b(id), _dp(d)))
        pt = Point(id, d)
        if self._obs_keys:
            errs, w, dims = self._projection_results()
            for k, (s, p) in enumerate(self._obs_keys):
                if p == id:
                    pt.reprojection_errors[s] = errs[k, : dims[k]].copy()
                    pt.reprojection_weights[s] = float(w[k])
        return pt

    def add_point_projection_observation(self, shot: str, point: str, observation, std_deviation: float,
                                         is_gcp: bool = False, depth_prior: Optional[Depth] = None) -> None:
        """AddPointProjectionObservation (bundle_adjuster.cc:274-287); a
        ``depth_prior`` (``Depth``: value, is_radial, std_deviation) adds a
        RelativeDepthError residual at run (:572-604); a non-finite value
        makes ``run`` raise RuntimeError, as the reference's Run does."""
        o = _vec(observation, 2)
        self._check(self._L.gbba_add_point_projection_observation(self._h, _b(shot), _b(point), _dp(o),
                                                                  float(std_deviation), int(is_gcp)))
        self._obs_keys.append((shot, point))
        if depth_prior is not None:
            n = int(self._L.gbba_num_projections(self._h))
            self.set_depth_priors([n - 1], [depth_prior.value], [depth_prior.std_deviation],
                                  [bool(depth_prior.is_radial)])

    def set_depth_priors(self, observation_index, value, std_deviation, is_radial=True) -> None:
        """Bulk form of ``depth_prior``: attaches depth priors to the
        observations of the given insertion indices (0-based, over every
        observation added so far)."""
        idx = np.ascontiguousarray(observation_index, np.int64).reshape(-1)
        n = len(idx)
        val = np.ascontiguousarray(np.broadcast_to(np.asarray(value, np.float64), (n,)))
        sd = np.ascontiguousarray(np.broadcast_to(np.asarray(std_deviation, np.float64), (n,)))
        rad = np.ascontiguousarray(np.broadcast_to(np.asarray(is_radial, np.uint8), (n,)))
        self._check(self._L.gbba_set_observation_depth_priors(
            self._h, n, idx.ctypes.data_as(C.POINTER(C.c_int64)), _dp(val), _dp(sd), rad.ctypes.data_as(_U8)))

    # -- bulk interface (raw-index path of BAHelpers) ----------------------
    def shot_index(self, shot: str) -> int:
        return int(self._L.gbba_shot_index(self._h, _b(shot)))

    def point_index(self, point: str) -> int:
        return int(self._L.gbba_point_index(self._h, _b(point)))

    def add_points(self, positions: np.ndarray, constant: Optional[np.ndarray] = None) -> int:
        """Adds points with ids "<index>"; returns the first index."""
        xyz = np.ascontiguousarray(positions, np.float64).reshape(-1, 3)
        c = None if constant is None else np.ascontiguousarray(constant, np.uint8)
        first = C.c_int64(0)
        self._check(self._L.gbba_add_points_bulk(self._h, len(xyz), _dp(xyz),
                                                  None if c is None else c.ctypes.data_as(_U8), None,
                                                  C.byref(first)))
        self._point_ids = None
        return int(first.value)

    def add_point_projection_observations(self, shot_index, point_index, observations, std_deviation,
                                          is_gcp=None) -> None:
        s = np.ascontiguousarray(shot_index, np.int32)
        p = np.ascontiguousarray(point_index, np.int32)
        xy = np.ascontiguousarray(observations, np.float64).reshape(-1, 2)
        sd = np.ascontiguousarray(np.broadcast_to(np.asarray(std_deviation, np.float64), (len(s),)))
        g = None if is_gcp is None else np.ascontiguousarray(is_gcp, np.uint8)
        self._check(self._L.gbba_add_point_projection_observations_bulk(
            self._h, len(s), s.ctypes.data_as(_I32), p.ctypes.data_as(_I32), _dp(xy), _dp(sd),
            None if g is None else g.ctypes.data_as(_U8)))
        self._obs_keys = []

    def get_points(self) -> np.ndarray:
        n = int(self._L.gbba_num_points(self._h))
        out = np.zeros((n, 3))
        self._check(self._L.gbba_get_points_bulk(self._h, 0, n, _dp(out)))
        return out

    def _projection_results(self):
        n = int(self._L.gbba_num_projections(self._h))
        errs = np.zeros((n, 3))
        w = np.zeros(n)
        dims = np.zeros(n, np.int32)
        self._check(self._L.gbba_get_projection_results(self._h, n, _dp(errs), _dp(w), dims.ctypes.data_as(_I32)))
        return errs, w, dims

    def add_absolute_up_vector(self, shot_id: str, up_vector, std_deviation: float) -> None:
        v = np.ascontiguousarray(up_vector, dtype=np.float64)
        self._check(self._L.gbba_add_absolute_up_vector(self._h, _b(shot_id), _dp(v), float(std_deviation)))

    def add_absolute_pan(self, shot_id: str, angle: float, std_deviation: float) -> None:
        self._check(self._L.gbba_add_absolute_pan(self._h, _b(shot_id), float(angle), float(std_deviation)))

    def add_absolute_tilt(self, shot_id: str, angle: float, std_deviation: float) -> None:
        self._check(self._L.gbba_add_absolute_tilt(self._h, _b(shot_id), float(angle), float(std_deviation)))

    def add_absolute_roll(self, shot_id: str, angle: float, std_deviation: float) -> None:
        self._check(self._L.gbba_add_absolute_roll(self._h, _b(shot_id), float(angle), float(std_deviation)))

    def add_relative_rotation(self, rr: "RelativeRotation") -> None:
        sm = np.ascontiguousarray(rr.scale_matrix, dtype=np.float64).reshape(9)
        r = _vec(rr.r, 3)
        self._check(self._L.gbba_add_relative_rotation(self._h, _b(rr.shot_i), _b(rr.shot_j), _dp(r), _dp(sm)))

    def add_common_position(self, shot_i: str, shot_j: str, margin: float, std_deviation: float) -> None:
        self._check(self._L.gbba_add_common_position(self._h, _b(shot_i), _b(shot_j), float(margin),
                                                     float(std_deviation)))

    def add_linear_motion(self, shot0: str, shot1: str, shot2: str, alpha: float, position_std_deviation: float,
                          orientation_std_deviation: float) -> None:
        self._check(self._L.gbba_add_linear_motion(self._h, _b(shot0), _b(shot1), _b(shot2), float(alpha),
                                                   float(position_std_deviation),
                                                   float(orientation_std_deviation)))

    def set_relative_motion_loss_function(self, name: str, threshold: float) -> None:
        self._check(self._L.gbba_set_relative_motion_loss_function(self._h, _b(name), float(threshold)))

    def add_heatmap(self, heatmap_id: str, in_heatmap, in_width: int, resolution: float) -> None:
        d = np.ascontiguousarray(np.asarray(in_heatmap, dtype=np.float64).reshape(-1))
        self._check(self._L.gbba_add_heatmap(self._h, _b(heatmap_id), _dp(d), d.size, int(in_width),
                                             float(resolution)))

    def add_absolute_position_heatmap(self, shot_id: str, heatmap_id: str, x_offset: float, y_offset: float,
                                      std_deviation: float) -> None:
        self._check(self._L.gbba_add_absolute_position_heatmap(self._h, _b(shot_id), _b(heatmap_id),
                                                               float(x_offset), float(y_offset),
                                                               float(std_deviation)))

    def add_reconstruction(self, reconstruction_id: str, constant: bool) -> None:
        self._check(self._L.gbba_add_reconstruction(self._h, _b(reconstruction_id), int(bool(constant))))

    def add_reconstruction_instance(self, reconstruction_id: str, scale: float, instance_id: str) -> None:
        self._check(self._L.gbba_add_reconstruction_instance(self._h, _b(reconstruction_id), float(scale),
                                                             _b(instance_id)))

    def set_scale_sharing(self, reconstruction_id: str, share: bool) -> None:
        self._check(self._L.gbba_set_scale_sharing(self._h, _b(reconstruction_id), int(bool(share))))

    def get_reconstruction(self, reconstruction_id: str) -> "Reconstruction":
        # the reference raises for an unknown id (bundle_adjuster.cc:1344-1350)
        if not self._L.gbba_has_reconstruction(self._h, _b(reconstruction_id)):
            raise RuntimeError(f"Reconstruction {reconstruction_id} doesn't exist.")
        return Reconstruction(self, reconstruction_id)

    def add_relative_motion(self, rm: "RelativeMotion") -> None:
        motion = np.ascontiguousarray(np.r_[rm.rotation, rm.translation, rm.scale], dtype=np.float64)
        sm = np.ascontiguousarray(rm.scale_matrix, dtype=np.float64).reshape(49)
        self._check(self._L.gbba_add_relative_motion(self._h, _b(rm.rig_instance_i), _b(rm.rig_instance_j),
                                                     _dp(motion), float(rm.robust_multiplier),
                                                     int(bool(rm.observed_scale)), _dp(sm)))

    def set_adjust_absolute_position_std(self, adjust: bool) -> None:
        self._check(self._L.gbba_set_adjust_absolute_position_std(self._h, int(bool(adjust))))

    def set_gauge_fix_shots(self, shot_origin: str, shot_scale: str) -> None:
        self._check(self._L.gbba_set_gauge_fix_shots(self._h, _b(shot_origin), _b(shot_scale)))

    def find_outliers(self, filter_type: str = "FIXED", fixed_threshold: float = 0.006, auto_ratio: float = 3.0,
                      weight_threshold: float = 0.5):
        """Outlier observations of the last solve, as sfm::BAHelpers::RemoveOutliers
        selects them (ba_helpers.cc:1847-1975), computed on the device.  Returns
        (threshold, outlier flags per observation, removed flags per point), both
        in insertion order."""
        from .outliers import adjuster_outliers
        return adjuster_outliers(self, filter_type=filter_type, fixed_threshold=fixed_threshold,
                                 auto_ratio=auto_ratio, weight_threshold=weight_threshold)

    def projection_results(self):
        """(errors [n, 3], weights [n], dims [n]) per observation in insertion order."""
        return self._projection_results()

    # -- settings -----------------------------------------------------------
    def set_point_projection_loss_function(self, name: str, threshold: float) -> None:
        self._check(self._L.gbba_set_point_projection_loss_function(self._h, _b(name), float(threshold)))

    def set_irls_mode(self, mode: str) -> None:
        self._check(self._L.gbba_set_irls_mode(self._h, {"none": 0, "mixture": 1}[mode]))

    def set_precision(self, precision: str) -> None:
        self._check(self._L.gbba_set_precision(self._h, {"fp64": 0, "mixed": 1}[precision]))

    def set_pcg_tolerance(self, tolerance: float) -> None:
        self._check(self._L.gbba_set_pcg_tolerance(self._h, float(tolerance)))

    def set_matrix_free(self, mode: int) -> None:
        """0: store the Jacobian records when they fit in device memory (the
        default), 1: evaluate them in every pass, -1: always store them."""
        self._check(self._L.gbba_set_matrix_free(self._h, int(mode)))

    def set_pcg_graph(self, enable: bool) -> None:
        """True (default): a linear solve's PCG iterations run as one CUDA
        graph launch; False: kernel by kernel (a profiler then sees every
        launch)."""
        self._check(self._L.gbba_set_pcg_graph(self._h, int(enable)))

    def set_coarse_preconditioner(self, leaf: int) -> None:
        """leaf > 0: two-level PCG preconditioner, block-Jacobi plus a coarse
        space of similarity modes over spatial clusters of at most `leaf` rig
        instances (include/gbba.h, gbba_set_coarse_preconditioner); 0 (the
        default): block-Jacobi only."""
        self._check(self._L.gbba_set_coarse_preconditioner(self._h, int(leaf)))

    def coarse_info(self) -> dict:
        """Clusters, colours and probe products of the last run's coarse space."""
        a, b, c = C.c_int(0), C.c_int(0), C.c_int64(0)
        self._check(self._L.gbba_get_coarse_info(self._h, C.byref(a), C.byref(b), C.byref(c)))
        return {"clusters": a.value, "colours": b.value, "probes": c.value}

    def coarse_space_layout(self, leaf: int, n_instances: int):
        """The coarse space the current problem would get (no solve): the
        cluster of every rig instance (insertion order, -1: none) and the
        colour of every cluster."""
        cl = np.zeros(n_instances, dtype=np.int32)
        col = np.zeros(max(1, n_instances), dtype=np.int32)
        nc, ncol = C.c_int(0), C.c_int(0)
        self._check(self._L.gbba_coarse_space_layout(
            self._h, int(leaf), cl.ctypes.data_as(C.POINTER(C.c_int)), int(n_instances),
            col.ctypes.data_as(C.POINTER(C.c_int)), int(len(col)), C.byref(nc), C.byref(ncol)))
        return cl, col[:nc.value].copy(), ncol.value

    def set_shard(self, rank: int, world_size: int, allreduce=None) -> None:
        """Makes this adjuster rank `rank` of a point-partitioned solve over
        `world_size` GPUs (include/gbba.h, gbba_set_shard).  `allreduce(data,
        op)` reduces the float64 numpy array `data` in place over the ranks
        (op REDUCE_SUM or REDUCE_MAX); torch_allreduce() makes one from a
        torch.distributed process group.  world_size 1 restores the
        single-GPU solve."""
        if world_size > 1 and allreduce is None:
            raise ValueError("a sharded solve needs an all-reduce")
        if world_size > 1:
            def _cb(ctx, data, count, op):
                try:
                    allreduce(np.ctypeslib.as_array(data, shape=(int(count),)), int(op))
                    return 0
                except Exception:  # reported to the solver as a failed collective
                    import traceback
                    traceback.print_exc()
                    return 1
            self._allreduce_cb = ALLREDUCE_FN(_cb)
        else:
            self._allreduce_cb = ALLREDUCE_FN()
        self._check(self._L.gbba_set_shard(self._h, int(rank), int(world_size), self._allreduce_cb, None))

    def shard_points(self, rank: int) -> tuple[int, int]:
        """Points [first, last) (insertion order) that `rank` solves with."""
        a, b = C.c_int64(0), C.c_int64(0)
        self._check(self._L.gbba_get_shard_points(self._h, int(rank), C.byref(a), C.byref(b)))
        return a.value, b.value

    def set_max_num_iterations(self, n: int) -> None:
        self._check(self._L.gbba_set_max_num_iterations(self._h, int(n)))

    def set_num_threads(self, n: int) -> None:
        self._check(self._L.gbba_set_num_threads(self._h, int(n)))

    def set_use_analytic_derivatives(self, use: bool) -> None:
        self._check(self._L.gbba_set_use_analytic_derivatives(self._h, int(use)))

    def set_linear_solver_type(self, t: str) -> None:
        self._check(self._L.gbba_set_linear_solver_type(self._h, _b(t)))

    def set_internal_parameters_prior_sd(self, focal_sd, aspect_ratio_sd, c_sd, k1_sd, k2_sd, p1_sd, p2_sd, k3_sd,
                                         k4_sd) -> None:
        self._check(self._L.gbba_set_internal_parameters_prior_sd(
            self._h, focal_sd, aspect_ratio_sd, c_sd, k1_sd, k2_sd, p1_sd, p2_sd, k3_sd, k4_sd))

    def set_rig_parameters_prior_sd(self, rig_translation_sd, rig_rotation_sd) -> None:
        self._check(self._L.gbba_set_rig_parameters_prior_sd(self._h, rig_translation_sd, rig_rotation_sd))

    def set_compute_reprojection_errors(self, v: bool) -> None:
        self._check(self._L.gbba_set_compute_reprojection_errors(self._h, int(v)))

    def set_compute_covariances(self, v: bool) -> None:
        self._check(self._L.gbba_set_compute_covariances(self._h, int(v)))

    def get_covariance_estimation_valid(self) -> bool:
        return bool(self._L.gbba_get_covariance_estimation_valid(self._h))

    def get_rig_instance_covariance(self, id: str) -> np.ndarray:
        """6 x 6 covariance of the rig instance's pose [rx ry rz tx ty tz]."""
        out = np.zeros((6, 6))
        self._check(self._L.gbba_get_rig_instance_covariance(self._h, _b(id), _dp(out)))
        return out

    def set_skip_initial_reweighting(self, v: bool) -> None:
        self._check(self._L.gbba_set_skip_initial_reweighting(self._h, int(v)))

    def set_default_density_ratio(self, r: float) -> None:
        self._check(self._L.gbba_set_default_density_ratio(self._h, float(r)))

    def get_default_density_ratio(self) -> float:
        return float(self._L.gbba_get_default_density_ratio(self._h))

    def set_group_density_ratio(self, group: str, r: float) -> None:
        self._check(self._L.gbba_set_group_density_ratio(self._h, _b(group), float(r)))

    def get_group_density_ratio(self, group: str) -> float:
        return float(self._L.gbba_get_group_density_ratio(self._h, _b(group)))

    # -- run and reports ----------------------------------------------------
    def run(self) -> None:
        self._check(self._L.gbba_run(self._h))

    def _report(self, fn) -> str:
        n = fn(self._h, None, 0)
        if n < 0:
            raise RuntimeError(self._L.gbba_last_error().decode())
        buf = C.create_string_buffer(n + 1)
        fn(self._h, buf, n + 1)
        return buf.value.decode("utf-8", "replace")

    def brief_report(self) -> str:
        return self._report(self._L.gbba_brief_report)

    def full_report(self) -> str:
        return self._report(self._L.gbba_full_report)

    def irls_report(self) -> list:
        text = self._report(self._L.gbba_irls_report)
        return text.split("\n") if text else []

    def summary(self) -> dict:
        s = Summary()
        self._check(self._L.gbba_get_summary(self._h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in Summary._fields_}

    def trace(self) -> np.ndarray:
        """Iteration records [iteration, cost, seconds, success, linear iterations,
        radius, relative decrease, step norm]."""
        n = C.c_int(0)
        self._check(self._L.gbba_get_trace(self._h, 0, None, C.byref(n)))
        out = np.zeros((n.value, 8))
        self._check(self._L.gbba_get_trace(self._h, n.value, _dp(out), C.byref(n)))
        return out


class BatchSummary(C.Structure):
    _fields_ = [("seconds", C.c_double), ("setup_seconds", C.c_double), ("solve_seconds", C.c_double),
                ("lm_iterations", C.c_int), ("grid", C.c_int), ("n_problems", C.c_int), ("n_converged", C.c_int),
                ("graph_nodes", C.c_int64), ("kernel_launches", C.c_int64), ("graph_launches", C.c_int64)]


class BundleBatch:
    """Many BundleAdjusters solved together on the GPU (gbba_batch_*).

    The reference solves one local bundle adjustment per call
    (sfm::BAHelpers::BundleLocal); a batch solves many of them in one device
    layout with per-problem trust regions, replaying one recorded LM
    iteration.  After run() every adjuster's getters and reports hold its
    own result."""

    def __init__(self) -> None:
        self._L = _lib.lib()
        _declare(self._L)
        L = self._L
        for name, args, res in (("gbba_batch_create", [], _H), ("gbba_batch_destroy", [_H], None),
                                ("gbba_batch_add", [_H, _H], C.c_int), ("gbba_batch_size", [_H], C.c_int),
                                ("gbba_batch_set_options", [_H, C.c_int, C.c_int, C.c_int, C.c_double, C.c_int,
                                                            C.c_int], C.c_int),
                                ("gbba_batch_run", [_H], C.c_int),
                                ("gbba_batch_set_function_tolerance", [_H, C.c_double], C.c_int),
                                ("gbba_batch_set_linear_solver", [_H, C.c_char_p], C.c_int),
                                ("gbba_batch_get_summary", [_H, C.POINTER(BatchSummary)], C.c_int)):
            f = getattr(L, name)
            f.argtypes = args
            f.restype = res
        self._h = L.gbba_batch_create()
        self._members: list = []  # keeps the adjusters alive while the batch refers to them

    def __del__(self) -> None:
        h = getattr(self, "_h", None)
        if h:
            self._L.gbba_batch_destroy(h)
            self._h = None

    def add(self, ba: BundleAdjuster) -> None:
        _lib.check(self._L.gbba_batch_add(self._h, ba._h))
        self._members.append(ba)

    def __len__(self) -> int:
        return int(self._L.gbba_batch_size(self._h))

    def set_options(self, precision: str = "mixed", max_iterations: int = 50, pcg_iterations: int = 50,
                    pcg_tolerance: float = 1e-3, use_graph: int = 2, autotune: bool = True) -> None:
        """use_graph 2: the whole LM loop one graph launch (device-side
        termination); 1: one graph launch per LM iteration; 0: plain
        launches."""
        p = {"fp64": _lib.PRECISION_FP64, "mixed": _lib.PRECISION_MIXED}[precision]
        _lib.check(self._L.gbba_batch_set_options(self._h, p, max_iterations, pcg_iterations, pcg_tolerance,
                                                  int(use_graph), int(autotune)))

    def set_function_tolerance(self, tolerance: float) -> None:
        _lib.check(self._L.gbba_batch_set_function_tolerance(self._h, tolerance))

    def set_linear_solver_type(self, name: str) -> None:
        """DENSE_SCHUR (or another exact type): every step exact, in FP64
        (PCG to a 1e-10 relative residual); ITERATIVE_SCHUR (the default):
        the options' precision and PCG."""
        _lib.check(self._L.gbba_batch_set_linear_solver(self._h, name.encode()))

    def run(self) -> None:
        _lib.check(self._L.gbba_batch_run(self._h))

    def summary(self) -> dict:
        s = BatchSummary()
        _lib.check(self._L.gbba_batch_get_summary(self._h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in BatchSummary._fields_}


ORIENTATION_KINDS = {"up_vector": 0, "pan": 1, "tilt": 2, "roll": 3}


def orientation_residual(kind: str, target, std_deviation: float, instance_rotation, camera_rotation=None):
    """Scaled residuals (before the loss) and Jacobian [m][6] of one absolute
    orientation constraint -- UpVectorError, PanAngleError, TiltAngleError
    or RollAngleError (bundle/error/absolute_motion_errors.h:10-126) -- at
    the given rig instance and rig camera rotations (angle-axis)."""
    L = _lib.lib()
    _declare(L)
    t = np.zeros(3)
    v = np.atleast_1d(np.asarray(target, dtype=np.float64))
    t[: len(v)] = v
    ri = np.ascontiguousarray(instance_rotation, dtype=np.float64)
    rc = None if camera_rotation is None else np.ascontiguousarray(camera_rotation, dtype=np.float64)
    r, J = np.zeros(3), np.zeros(18)
    m = C.c_int(0)
    _lib.check(L.gbba_orientation_residual(ORIENTATION_KINDS[kind], _dp(t), float(std_deviation), _dp(ri),
                                           _dp(rc) if rc is not None else None, _dp(r), _dp(J), C.byref(m)))
    return r[: m.value].copy(), J[: 6 * m.value].reshape(m.value, 6)


RELATIVE_KINDS = {"relative_rotation": 0, "common_position": 1, "linear_motion": 2, "gauge_scale": 3,
                  "relative_motion": 5, "gps_std": 6, "std_deviation": 7, "gps_bias": 8}


def relative_residual(kind: str, instance_poses, params, rig_camera_poses=None):
    """Scaled residuals (before the loss) and Jacobian [m][36] of one host
    constraint -- RelativeRotationError, CommonPositionError
    (relative_motion_errors.h:66-126), LinearMotionError
    (motion_prior_errors.h:12-74), the gauge scale, RelativeMotionError, the
    std-adjusted GPS prior (prior_error.h:54-93) or StdDeviationConstraint
    (parameters_errors.h:7-16).  Poses [n][6] as [rx ry rz tx ty tz] with t
    the position (None for the std regulariser); params as
    gbba_relative_residual takes them ("gps_bias": the GPS prior through an
    optimised camera bias, prior[3], std[3], multiplier, bias[7])."""
    L = _lib.lib()
    _declare(L)
    pi = None if instance_poses is None else np.ascontiguousarray(instance_poses, dtype=np.float64)
    pc = None if rig_camera_poses is None else np.ascontiguousarray(rig_camera_poses, dtype=np.float64)
    prm = np.ascontiguousarray(params, dtype=np.float64).reshape(-1)
    r, J = np.zeros(7), np.zeros(7 * 36)
    m = C.c_int(0)
    _lib.check(L.gbba_relative_residual(RELATIVE_KINDS[kind], _dp(pi) if pi is not None else None,
                                        _dp(pc) if pc is not None else None,
                                        _dp(prm), _dp(r), _dp(J), C.byref(m)))
    return r[: m.value].copy(), J[: 36 * m.value].reshape(m.value, 36)


def heatmap_residual(grid, width: int, resolution: float, x_offset: float, y_offset: float, std_deviation: float,
                     instance_pose, rig_camera_pose=None):
    """HeatmapdCostFunctor (absolute_motion_errors.h:128-173): the residual
    and its Jacobian [12] at the given instance and rig camera poses."""
    L = _lib.lib()
    _declare(L)
    g = np.ascontiguousarray(np.asarray(grid, dtype=np.float64).reshape(-1))
    pi = np.ascontiguousarray(instance_pose, dtype=np.float64)
    pc = None if rig_camera_pose is None else np.ascontiguousarray(rig_camera_pose, dtype=np.float64)
    r, J = np.zeros(1), np.zeros(12)
    _lib.check(L.gbba_heatmap_residual(_dp(g), g.size, int(width), float(resolution), float(x_offset),
                                       float(y_offset), float(std_deviation), _dp(pi),
                                       _dp(pc) if pc is not None else None, _dp(r), _dp(J)))
    return float(r[0]), J


def adjuster_from_scene(scene, precision: str = "mixed", loss: Optional[tuple] = None, irls: str = "mixture",
                        gps: bool = True, constant_cameras: bool = False, max_iterations: int = 100,
                        pcg_tolerance: Optional[float] = None, linear_solver: Optional[str] = None,
                        matrix_free: Optional[int] = None, covariances: bool = False, depth=None,
                        rig_pose=None, bias=None, point_priors=None, pcg_graph: bool = True,
                        coarse_leaf: int = 0, fixed_instances=None) -> BundleAdjuster:
    """Builds a BundleAdjuster from a SceneArrays (bulk path).  ``depth``:
    depth priors (observation indices, values, stds, radial flags);
    ``rig_pose``: a fixed rig camera pose (angle-axis, centre) shared by every
    shot (None: the identity); ``bias``: (rotation, translation, scale,
    parameters to optimise) of every camera's bias; ``point_priors``: (point
    indices, positions, stds) with altitude; ``coarse_leaf``: the two-level
    preconditioner's cluster size (0: block-Jacobi only); ``fixed_instances``:
    rig instance indices added as constant."""
    ba = BundleAdjuster()
    ba.set_precision(precision)
    if not pcg_graph:
        ba.set_pcg_graph(False)
    if coarse_leaf:
        ba.set_coarse_preconditioner(coarse_leaf)
    if matrix_free is not None:
        ba.set_matrix_free(matrix_free)
    if covariances:
        ba.set_compute_covariances(True)
    if linear_solver is not None:
        ba.set_linear_solver_type(linear_solver)
    ba.set_irls_mode(irls)
    ba.set_max_num_iterations(max_iterations)
    if pcg_tolerance is not None:
        ba.set_pcg_tolerance(pcg_tolerance)
    if loss is not None:
        ba.set_point_projection_loss_function(*loss)
    for c in range(len(scene.camera_projection)):
        m = int(scene.camera_projection[c])
        from .scene import NUM_PARAMS
        cam = Camera(m, scene.camera_values[c, : NUM_PARAMS[m]])
        ba.add_camera(str(c), cam, cam, constant_cameras)
    fixed = set() if fixed_instances is None else {int(i) for i in fixed_instances}
    rp = Pose() if rig_pose is None else Pose.from_ba_data(np.asarray(rig_pose, np.float64))
    ba.add_rig_camera("rig", rp, rp, True)
    for s in range(len(scene.shot_camera)):
        inst = int(scene.shot_rig_instance[s])
        pose = Pose.from_ba_data(scene.rig_instance_poses[inst])
        ba.add_rig_instance(str(inst), pose, {str(s): str(int(scene.shot_camera[s]))}, {str(s): "rig"},
                            inst in fixed)
    if gps and "gps" in scene.extras:
        for s in range(len(scene.shot_camera)):
            ba.add_rig_instance_position_prior(str(int(scene.shot_rig_instance[s])), scene.extras["gps"][s],
                                               scene.extras["gps_std"][s], "")
    if bias is not None:
        for c in range(len(scene.camera_projection)):
            ba.set_camera_bias(str(c), Similarity(bias[0], bias[1], bias[2]), bias[3])
    ba.add_points(scene.points)
    if point_priors is not None:
        for k, pos, sd in zip(np.asarray(point_priors[0]), np.asarray(point_priors[1]), np.asarray(point_priors[2])):
            ba.add_point_prior(str(int(k)), pos, sd, True)
    ba.add_point_projection_observations(scene.obs_shot, scene.obs_point, scene.obs_xy, scene.obs_std)
    if depth is not None:
        ba.set_depth_priors(*depth)
    return ba


__all__ = ["BundleAdjuster", "BundleBatch", "Depth", "Point", "Reconstruction", "RelativeMotion", "RelativeRotation",
           "adjuster_from_scene",
           "heatmap_residual", "orientation_residual", "relative_residual"]
