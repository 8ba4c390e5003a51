"""Flat-array bundle-adjustment scene, the Python side of ``gbba_scene_t``.

A :class:`SceneArrays` holds cameras, rig instances (shot poses), rig
cameras, shots, points and observations as numpy arrays in the layout of the
C ABI (include/gbba.h).  Poses are camera-to-world ``[rx, ry, rz, tx, ty,
tz]`` (angle-axis, camera centre) as bundle::Pose stores them
(opensfm/src/lib/bundle/data/pose.h:17,34-43); camera parameter vectors
follow geometry::Camera (opensfm/src/lib/geometry/src/camera.cc:11-172),
padded to 16 values.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _lib

MAX_CAMERA_PARAMS = 16

PERSPECTIVE, BROWN, FISHEYE, FISHEYE_OPENCV, FISHEYE62, FISHEYE624, SPHERICAL, DUAL, RADIAL, \
    SIMPLE_RADIAL = range(10)

NUM_PARAMS = {PERSPECTIVE: 3, BROWN: 9, FISHEYE: 3, FISHEYE_OPENCV: 8, FISHEYE62: 12,
              FISHEYE624: 16, SPHERICAL: 1, DUAL: 4, RADIAL: 6, SIMPLE_RADIAL: 5}


@dataclass
class SceneArrays:
    camera_projection: np.ndarray          # int32 [nc]
    camera_values: np.ndarray              # float64 [nc, 16]
    rig_instance_poses: np.ndarray         # float64 [ni, 6]
    shot_rig_instance: np.ndarray          # int32 [ns]
    shot_camera: np.ndarray                # int32 [ns]
    points: np.ndarray                     # float64 [np, 3]
    obs_shot: np.ndarray                   # int32 [no]
    obs_point: np.ndarray                  # int32 [no]
    obs_xy: np.ndarray                     # float64 [no, 2]
    obs_std: np.ndarray                    # float64 [no]
    rig_camera_poses: np.ndarray = field(default_factory=lambda: np.zeros((0, 6)))
    rig_camera_used: np.ndarray = field(default_factory=lambda: np.zeros((0,), np.uint8))
    shot_rig_camera: np.ndarray | None = None  # int32 [ns], -1: no rig camera
    extras: dict = field(default_factory=dict)

    def __post_init__(self) -> None:
        self.camera_projection = np.ascontiguousarray(self.camera_projection, np.int32)
        cv = np.zeros((len(self.camera_projection), MAX_CAMERA_PARAMS))
        v = np.asarray(self.camera_values, np.float64)
        cv[:, : v.shape[1]] = v
        self.camera_values = cv
        self.rig_instance_poses = np.ascontiguousarray(self.rig_instance_poses, np.float64).reshape(-1, 6)
        self.shot_rig_instance = np.ascontiguousarray(self.shot_rig_instance, np.int32)
        self.shot_camera = np.ascontiguousarray(self.shot_camera, np.int32)
        if self.shot_rig_camera is None:
            self.shot_rig_camera = np.full(len(self.shot_camera), -1, np.int32)
        self.shot_rig_camera = np.ascontiguousarray(self.shot_rig_camera, np.int32)
        self.rig_camera_poses = np.ascontiguousarray(self.rig_camera_poses, np.float64).reshape(-1, 6)
        self.rig_camera_used = np.ascontiguousarray(self.rig_camera_used, np.uint8)
        self.points = np.ascontiguousarray(self.points, np.float64).reshape(-1, 3)
        self.obs_shot = np.ascontiguousarray(self.obs_shot, np.int32)
        self.obs_point = np.ascontiguousarray(self.obs_point, np.int32)
        self.obs_xy = np.ascontiguousarray(self.obs_xy, np.float64).reshape(-1, 2)
        self.obs_std = np.ascontiguousarray(self.obs_std, np.float64)

    @property
    def n_observations(self) -> int:
        return len(self.obs_shot)

    def ctypes(self) -> _lib.Scene:
        """A ``gbba_scene_t`` viewing these arrays (keep self alive)."""
        s = _lib.Scene()
        s.n_cameras = len(self.camera_projection)
        s.camera_projection = _lib._ptr(self.camera_projection, C.c_int32)
        s.camera_values = _lib._ptr(self.camera_values, C.c_double)
        s.n_rig_instances = len(self.rig_instance_poses)
        s.rig_instance_poses = _lib._ptr(self.rig_instance_poses, C.c_double)
        s.n_rig_cameras = len(self.rig_camera_poses)
        s.rig_camera_poses = _lib._ptr(self.rig_camera_poses, C.c_double)
        s.rig_camera_used = _lib._ptr(self.rig_camera_used, C.c_uint8)
        s.n_shots = len(self.shot_camera)
        s.shot_rig_instance = _lib._ptr(self.shot_rig_instance, C.c_int32)
        s.shot_rig_camera = _lib._ptr(self.shot_rig_camera, C.c_int32)
        s.shot_camera = _lib._ptr(self.shot_camera, C.c_int32)
        s.n_points = len(self.points)
        s.points = _lib._ptr(self.points, C.c_double)
        s.n_observations = len(self.obs_shot)
        s.obs_shot = _lib._ptr(self.obs_shot, C.c_int32)
        s.obs_point = _lib._ptr(self.obs_point, C.c_int32)
        s.obs_xy = _lib._ptr(self.obs_xy, C.c_double)
        s.obs_std = _lib._ptr(self.obs_std, C.c_double)
        return s

    def layout(self) -> tuple[int, int]:
        """(nr, cmax) of the evaluation outputs."""
        used = np.unique(self.shot_camera)
        models = self.camera_projection[used] if len(used) else np.array([], np.int32)
        nr = 3 if np.any(models == SPHERICAL) else 2
        cmax = max([1] + [NUM_PARAMS[int(m)] for m in models])
        return nr, cmax

    def subset_observations(self, idx: np.ndarray) -> "SceneArrays":
        """Same scene restricted to the observations idx."""
        out = SceneArrays(self.camera_projection, self.camera_values, self.rig_instance_poses,
                          self.shot_rig_instance, self.shot_camera, self.points,
                          self.obs_shot[idx], self.obs_point[idx], self.obs_xy[idx],
                          self.obs_std[idx], self.rig_camera_poses, self.rig_camera_used,
                          self.shot_rig_camera)
        return out


@dataclass
class EvalResult:
    residuals: np.ndarray
    jac_camera: np.ndarray
    jac_instance: np.ndarray
    jac_rig_camera: np.ndarray
    jac_point: np.ndarray


def alloc_outputs(n: int, nr: int, cmax: int, pinned=None) -> EvalResult:
    mk = pinned or (lambda shape: np.zeros(shape))
    return EvalResult(mk((n, nr)), mk((n, nr, cmax)), mk((n, nr, 6)), mk((n, nr, 6)), mk((n, nr, 3)))


def output_struct(r: EvalResult) -> _lib.EvalOutput:
    o = _lib.EvalOutput()
    o.residuals = _lib._ptr(r.residuals, C.c_double)
    o.jac_camera = _lib._ptr(r.jac_camera, C.c_double)
    o.jac_instance = _lib._ptr(r.jac_instance, C.c_double)
    o.jac_rig_camera = _lib._ptr(r.jac_rig_camera, C.c_double)
    o.jac_point = _lib._ptr(r.jac_point, C.c_double)
    return o


def evaluate_projections(scene: SceneArrays, precision: int = _lib.PRECISION_FP64) -> EvalResult:
    """Residuals and Jacobian blocks of every observation, evaluated on the GPU."""
    L = _lib.lib()
    nr, cmax = scene.layout()
    out = alloc_outputs(scene.n_observations, nr, cmax)
    s = scene.ctypes()
    o = output_struct(out)
    _lib.check(L.gbba_evaluate_projections(C.byref(s), precision, C.byref(o)))
    return out


class Evaluator:
    """Device-resident evaluator (``gbba_evaluator_*``)."""

    def __init__(self, scene: SceneArrays, precision: int = _lib.PRECISION_MIXED):
        self._L = _lib.lib()
        self.scene = scene
        s = scene.ctypes()
        h = self._L.gbba_evaluator_create(C.byref(s), precision)
        if not h:
            self._h = None
            raise _lib.GbbaError(_lib.GBBA_ERR_RUNTIME,
                                 self._L.gbba_last_error().decode("utf-8", "replace"))
        self._h = h

    def run(self, stream: int | None = None) -> None:
        _lib.check(self._L.gbba_evaluator_run(self._h, C.c_void_p(stream or 0)))

    def prepare(self, stream: int | None = None) -> None:
        _lib.check(self._L.gbba_evaluator_prepare(self._h, C.c_void_p(stream or 0)))

    def records(self, stream: int | None = None) -> None:
        _lib.check(self._L.gbba_evaluator_records(self._h, C.c_void_p(stream or 0)))

    def download(self) -> EvalResult:
        nr, cmax = self.scene.layout()
        out = alloc_outputs(self.scene.n_observations, nr, cmax)
        o = output_struct(out)
        _lib.check(self._L.gbba_evaluator_download(self._h, C.byref(o)))
        return out

    @property
    def launches_per_run(self) -> int:
        return int(self._L.gbba_evaluator_launches_per_run(self._h))

    @property
    def record_bytes(self) -> int:
        return int(self._L.gbba_evaluator_record_bytes(self._h))

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._L.gbba_evaluator_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()
