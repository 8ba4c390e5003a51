"""Projection + residual as a differentiable PyTorch operator.

``project_residuals(...)`` returns the scaled reprojection residuals
r_i = (pi(camera, pose, X) - obs_i) / std_i of every observation (the
residual of ReprojectionError2DAnalytic<C>, opensfm/src/lib/bundle/error/
projection_errors.h:67-207, with the shot pose equal to its rig instance's)
and differentiates them with respect to the camera parameter vectors, the
instance poses [rx ry rz tx ty tz] and the points.  Forward and backward
are the hand-written CUDA kernels of libgbba.so (gbba_projection_forward /
gbba_projection_backward); the backward contracts the analytic Jacobian
with the incoming gradient.

Two memory modes:
  stored     the forward saves the Jacobian records (16-byte planes) and the
             backward reads them;
  recompute  nothing per observation is kept; the backward evaluates the
             Jacobian again (matrix-free).
Both compute in the dtype of the inputs (float32 or float64).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Optional

import torch

from . import _lib

DTYPE_F64 = 0
DTYPE_F32 = 1
MAX_CAMERA_PARAMS = 16


class DeviceProblem(C.Structure):
    """Mirror of ``gbba_device_problem_t``."""

    _fields_ = [
        ("dtype", C.c_int32), ("model_hint", C.c_int32),
        ("n_cameras", C.c_int32), ("camera_projection", C.c_void_p), ("camera_values", C.c_void_p),
        ("n_instances", C.c_int32), ("instance_poses", C.c_void_p),
        ("n_points", C.c_int64), ("points", C.c_void_p),
        ("n_shots", C.c_int32), ("shot_instance", C.c_void_p), ("shot_camera", C.c_void_p),
        ("n_observations", C.c_int64), ("obs_shot", C.c_void_p), ("obs_point", C.c_void_p),
        ("obs_xy", C.c_void_p), ("obs_std", C.c_void_p),
    ]


def _declare(L) -> None:
    if getattr(L, "_gbba_autograd_declared", False):
        return
    P = C.POINTER(DeviceProblem)
    L.gbba_projection_scratch_bytes.argtypes = [P, C.POINTER(C.c_int64)]
    L.gbba_projection_record_bytes.argtypes = [P, C.POINTER(C.c_int64)]
    L.gbba_projection_forward.argtypes = [P, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    L.gbba_projection_backward.argtypes = [P, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                           C.c_void_p, C.c_void_p]
    for name in ("gbba_projection_scratch_bytes", "gbba_projection_record_bytes", "gbba_projection_forward",
                 "gbba_projection_backward"):
        getattr(L, name).restype = C.c_int
    L._gbba_autograd_declared = True


def _ptr(t: Optional[torch.Tensor]):
    return C.c_void_p(t.data_ptr()) if t is not None else C.c_void_p(None)


@dataclass
class Observations:
    """The non-differentiable part of a problem (device tensors)."""
    camera_projection: torch.Tensor  # int32 [nc]
    shot_instance: torch.Tensor      # int32 [ns]
    shot_camera: torch.Tensor        # int32 [ns]
    obs_shot: torch.Tensor           # int32 [no]
    obs_point: torch.Tensor          # int32 [no]
    obs_xy: torch.Tensor             # [no, 2]
    obs_std: torch.Tensor            # [no]
    model_hint: int = -1             # the single camera model, or -1


def _problem(obs: Observations, cams: torch.Tensor, poses: torch.Tensor, points: torch.Tensor) -> DeviceProblem:
    for name, t in (("camera_values", cams), ("instance_poses", poses), ("points", points), ("obs_xy", obs.obs_xy),
                    ("obs_std", obs.obs_std)):
        if not t.is_cuda or not t.is_contiguous():
            raise ValueError(f"{name} must be a contiguous CUDA tensor")
        if t.dtype != cams.dtype:
            raise TypeError(f"{name} has dtype {t.dtype}, expected {cams.dtype}")
    for name in ("camera_projection", "shot_instance", "shot_camera", "obs_shot", "obs_point"):
        t = getattr(obs, name)
        if not t.is_cuda or t.dtype != torch.int32 or not t.is_contiguous():
            raise ValueError(f"{name} must be a contiguous int32 CUDA tensor")
    if cams.dtype not in (torch.float32, torch.float64):
        raise TypeError("float32 or float64 tensors expected")
    if cams.shape[-1] != MAX_CAMERA_PARAMS or poses.shape[-1] != 6 or points.shape[-1] != 3:
        raise ValueError("camera_values [nc, 16], instance_poses [ni, 6], points [np, 3] expected")
    p = DeviceProblem()
    p.dtype = DTYPE_F64 if cams.dtype == torch.float64 else DTYPE_F32
    p.model_hint = int(obs.model_hint)
    p.n_cameras = int(cams.shape[0])
    p.camera_projection = _ptr(obs.camera_projection)
    p.camera_values = _ptr(cams)
    p.n_instances = int(poses.shape[0])
    p.instance_poses = _ptr(poses)
    p.n_points = int(points.shape[0])
    p.points = _ptr(points)
    p.n_shots = int(obs.shot_camera.shape[0])
    p.shot_instance = _ptr(obs.shot_instance)
    p.shot_camera = _ptr(obs.shot_camera)
    p.n_observations = int(obs.obs_shot.shape[0])
    p.obs_shot = _ptr(obs.obs_shot)
    p.obs_point = _ptr(obs.obs_point)
    p.obs_xy = _ptr(obs.obs_xy)
    p.obs_std = _ptr(obs.obs_std)
    return p


class _ProjectionResidual(torch.autograd.Function):
    @staticmethod
    def forward(ctx, camera_values, instance_poses, points, obs: Observations, recompute: bool):
        L = _lib.lib()
        _declare(L)
        cams = camera_values.detach().contiguous()
        poses = instance_poses.detach().contiguous()
        pts = points.detach().contiguous()
        p = _problem(obs, cams, poses, pts)
        nbytes = C.c_int64(0)
        _lib.check(L.gbba_projection_scratch_bytes(C.byref(p), C.byref(nbytes)))
        scratch = torch.empty(nbytes.value, dtype=torch.uint8, device=cams.device)
        records = None
        if not recompute:
            _lib.check(L.gbba_projection_record_bytes(C.byref(p), C.byref(nbytes)))
            records = torch.empty(max(nbytes.value, 16), dtype=torch.uint8, device=cams.device)
        res = torch.empty((p.n_observations, 2), dtype=cams.dtype, device=cams.device)
        stream = torch.cuda.current_stream(cams.device).cuda_stream
        _lib.check(L.gbba_projection_forward(C.byref(p), _ptr(res), _ptr(records), _ptr(scratch),
                                             C.c_void_p(stream)))
        ctx.obs = obs
        ctx.recompute = recompute
        ctx.save_for_backward(cams, poses, pts, scratch, records if records is not None else scratch)
        ctx.has_records = records is not None
        return res

    @staticmethod
    def backward(ctx, grad_res):
        L = _lib.lib()
        cams, poses, pts, scratch, records = ctx.saved_tensors
        if not ctx.has_records:
            records = None
        p = _problem(ctx.obs, cams, poses, pts)
        g = grad_res.contiguous().to(cams.dtype)
        gc = torch.zeros_like(cams) if ctx.needs_input_grad[0] else None
        gp = torch.zeros_like(poses) if ctx.needs_input_grad[1] else None
        gx = torch.zeros_like(pts) if ctx.needs_input_grad[2] else None
        stream = torch.cuda.current_stream(cams.device).cuda_stream
        _lib.check(L.gbba_projection_backward(C.byref(p), _ptr(g), _ptr(records), _ptr(scratch), _ptr(gc), _ptr(gp),
                                              _ptr(gx), C.c_void_p(stream)))
        return gc, gp, gx, None, None


def project_residuals(camera_values: torch.Tensor, instance_poses: torch.Tensor, points: torch.Tensor,
                      obs: Observations, recompute: bool = False) -> torch.Tensor:
    """Residuals [n_obs, 2] of every observation, differentiable with respect
    to camera_values [nc, 16], instance_poses [ni, 6] and points [np, 3]."""
    return _ProjectionResidual.apply(camera_values, instance_poses, points, obs, recompute)


def observations_from_scene(scene, dtype=torch.float64, device="cuda") -> tuple:
    """(camera_values, instance_poses, points, Observations) device tensors
    of a scene (opensfm_gb300.scene.SceneArrays) whose shots have no rig
    camera."""
    import numpy as np
    if scene.shot_rig_camera is not None and np.any(scene.shot_rig_camera >= 0):
        raise ValueError("the projection operator takes shots without rig cameras")
    models = np.unique(scene.camera_projection[np.unique(scene.shot_camera)])
    hint = int(models[0]) if len(models) == 1 else -1

    def f(a):
        return torch.as_tensor(np.ascontiguousarray(a), dtype=dtype, device=device)

    def i(a):
        return torch.as_tensor(np.ascontiguousarray(a, dtype=np.int32), device=device)

    obs = Observations(i(scene.camera_projection), i(scene.shot_rig_instance), i(scene.shot_camera),
                       i(scene.obs_shot), i(scene.obs_point), f(scene.obs_xy), f(scene.obs_std), hint)
    return f(scene.camera_values), f(scene.rig_instance_poses), f(scene.points), obs
