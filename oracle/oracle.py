"""ctypes wrapper of the FP64 CPU oracle (test infrastructure only).

Only tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` use this module, always as the checker or the timed CPU
baseline -- never as part of the product path.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

_LIB = Path(__file__).resolve().parent / "_build" / "liboracle.so"
_lib = None

D = C.POINTER(C.c_double)


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not _LIB.exists():
            from opensfm_gb300.build import build_oracle
            build_oracle()
        L = C.CDLL(str(_LIB))
        L.oracle_num_params.argtypes = [C.c_int]
        for name in ("oracle_project", "oracle_project_ad"):
            getattr(L, name).argtypes = [C.c_int, D, D, D, D, D]
            getattr(L, name).restype = None
        for name in ("oracle_residual_jacobian", "oracle_residual_ad"):
            getattr(L, name).argtypes = [C.c_int, D, D, D, D, D, C.c_double, D, D, D, D, D]
            getattr(L, name).restype = None
        L.oracle_evaluate_scene.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, D, D, D, D, D]
        for name in ("oracle_pose_jacobian", "oracle_pose_ad"):
            getattr(L, name).argtypes = [D, D, D, D]
            getattr(L, name).restype = None
        L.oracle_loss.argtypes = [C.c_int, C.c_double, C.c_double, D]
        L.oracle_loss.restype = None
        _declare_solver(L)
        _lib = L
    return _lib


def _declare_solver(L) -> None:
    if hasattr(L, "oracle_solve"):
        L.oracle_solve.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        L.oracle_solve.restype = C.c_int


def _p(a: np.ndarray | None):
    if a is None:
        return D()
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(D)


def num_params(model: int) -> int:
    return int(lib().oracle_num_params(model))


def project(model: int, p, params, ad: bool = False):
    """(uv, J wrt camera-frame point 2x3, J wrt params 2xC)."""
    c = num_params(model)
    p = np.ascontiguousarray(p, np.float64)
    prm = np.zeros(16)
    prm[: len(params)] = params
    uv, jp, jc = np.zeros(2), np.zeros(6), np.zeros(2 * c)
    fn = lib().oracle_project_ad if ad else lib().oracle_project
    fn(model, _p(p), _p(prm), _p(uv), _p(jp), _p(jc))
    return uv, jp.reshape(2, 3), jc.reshape(2, c)


def residual_jacobian(model: int, cam, inst, rig, X, obs, std: float, ad: bool = False):
    """(r, J_camera, J_instance, J_rig_camera, J_point) of one observation."""
    c = num_params(model)
    nr = 3 if model == 6 else 2
    cam_a = np.zeros(16)
    cam_a[: len(cam)] = cam
    args = [np.ascontiguousarray(x, np.float64) for x in (inst, X, obs)]
    rig_a = None if rig is None else np.ascontiguousarray(rig, np.float64)
    r, jc, ji, jr, jp = np.zeros(nr), np.zeros(nr * c), np.zeros(nr * 6), np.zeros(nr * 6), np.zeros(nr * 3)
    fn = lib().oracle_residual_ad if ad else lib().oracle_residual_jacobian
    fn(model, _p(cam_a), _p(args[0]), _p(rig_a), _p(args[1]), _p(args[2]), std, _p(r), _p(jc), _p(ji),
       _p(jr), _p(jp))
    return r, jc.reshape(nr, c), ji.reshape(nr, 6), jr.reshape(nr, 6), jp.reshape(nr, 3)


def evaluate_scene(scene, threads: int | None = None):
    """Oracle residuals / Jacobian blocks of every observation, laid out as
    gbba_evaluate_projections returns them."""
    from opensfm_gb300.scene import alloc_outputs, output_struct  # noqa: F401
    nr, cmax = scene.layout()
    n = scene.n_observations
    res, jc, ji, jr, jp = (np.zeros((n, nr)), np.zeros((n, nr, cmax)), np.zeros((n, nr, 6)),
                           np.zeros((n, nr, 6)), np.zeros((n, nr, 3)))
    s = scene.ctypes()
    threads = threads or os.cpu_count() or 1
    lib().oracle_evaluate_scene(C.addressof(s), nr, cmax, threads, _p(res), _p(jc), _p(ji), _p(jr), _p(jp))
    return res, jc, ji, jr, jp


def pose_jacobian(X, rt, ad: bool = False):
    """(x_cam, 3x9 Jacobian [dX | d r | d t]) of PoseFunctor."""
    X = np.ascontiguousarray(X, np.float64)
    rt = np.ascontiguousarray(rt, np.float64)
    out, J = np.zeros(3), np.zeros(27)
    fn = lib().oracle_pose_ad if ad else lib().oracle_pose_jacobian
    fn(_p(X), _p(rt), _p(out), _p(J))
    return out, J.reshape(3, 9)


def loss(kind: int, threshold: float, s: float):
    rho = np.zeros(3)
    lib().oracle_loss(kind, threshold, s, _p(rho))
    return rho
