"""ctypes binding of ``libgbba.so`` (the C ABI declared in include/gbba.h).

The library is built in-tree by :mod:`opensfm_gb300.build`.  There is no
fallback: if the shared library is missing or does not load, every entry
point raises.
"""
from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

import numpy as np

_LIB_PATH = Path(__file__).resolve().parent / "libgbba.so"
_lib = None
_lock = threading.Lock()

GBBA_OK = 0
GBBA_ERR_INVALID_ARGUMENT = 1
GBBA_ERR_RUNTIME = 2
GBBA_ERR_OUT_OF_RANGE = 3
GBBA_ERR_CUDA = 4
GBBA_ERR_INTERNAL = 5

PRECISION_FP64 = 0
PRECISION_MIXED = 1


class GbbaError(RuntimeError):
    """Error returned by the native library."""

    def __init__(self, status: int, message: str):
        super().__init__(message)
        self.status = status


class Scene(C.Structure):
    """Mirror of ``gbba_scene_t``."""

    _fields_ = [
        ("n_cameras", C.c_int32),
        ("camera_projection", C.POINTER(C.c_int32)),
        ("camera_values", C.POINTER(C.c_double)),
        ("n_rig_instances", C.c_int32),
        ("rig_instance_poses", C.POINTER(C.c_double)),
        ("n_rig_cameras", C.c_int32),
        ("rig_camera_poses", C.POINTER(C.c_double)),
        ("rig_camera_used", C.POINTER(C.c_uint8)),
        ("n_shots", C.c_int32),
        ("shot_rig_instance", C.POINTER(C.c_int32)),
        ("shot_rig_camera", C.POINTER(C.c_int32)),
        ("shot_camera", C.POINTER(C.c_int32)),
        ("n_points", C.c_int64),
        ("points", C.POINTER(C.c_double)),
        ("n_observations", C.c_int64),
        ("obs_shot", C.POINTER(C.c_int32)),
        ("obs_point", C.POINTER(C.c_int32)),
        ("obs_xy", C.POINTER(C.c_double)),
        ("obs_std", C.POINTER(C.c_double)),
    ]


class EvalOutput(C.Structure):
    """Mirror of ``gbba_eval_output_t``."""

    _fields_ = [
        ("residuals", C.POINTER(C.c_double)),
        ("jac_camera", C.POINTER(C.c_double)),
        ("jac_instance", C.POINTER(C.c_double)),
        ("jac_rig_camera", C.POINTER(C.c_double)),
        ("jac_point", C.POINTER(C.c_double)),
    ]


def _ptr(a: np.ndarray | None, ctype):
    if a is None:
        return C.POINTER(ctype)()
    return a.ctypes.data_as(C.POINTER(ctype))


def lib() -> C.CDLL:
    """Loads libgbba.so (raises if it has not been built)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not _LIB_PATH.exists():
            raise ImportError(
                f"{_LIB_PATH} is missing: build it with `python -m opensfm_gb300.build` "
                "(the bundle adjuster has no CPU fallback)")
        L = C.CDLL(str(_LIB_PATH))
        L.gbba_last_error.restype = C.c_char_p
        L.gbba_camera_num_params.argtypes = [C.c_int]
        L.gbba_scene_layout.argtypes = [C.POINTER(Scene), C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L.gbba_evaluate_projections.argtypes = [C.POINTER(Scene), C.c_int, C.POINTER(EvalOutput)]
        L.gbba_evaluator_create.argtypes = [C.POINTER(Scene), C.c_int]
        L.gbba_evaluator_create.restype = C.c_void_p
        L.gbba_evaluator_destroy.argtypes = [C.c_void_p]
        L.gbba_evaluator_destroy.restype = None
        L.gbba_evaluator_run.argtypes = [C.c_void_p, C.c_void_p]
        L.gbba_evaluator_prepare.argtypes = [C.c_void_p, C.c_void_p]
        L.gbba_evaluator_records.argtypes = [C.c_void_p, C.c_void_p]
        L.gbba_evaluator_download.argtypes = [C.c_void_p, C.POINTER(EvalOutput)]
        L.gbba_evaluator_launches_per_run.argtypes = [C.c_void_p]
        L.gbba_evaluator_record_bytes.argtypes = [C.c_void_p]
        L.gbba_evaluator_record_bytes.restype = C.c_int64
        _declare_adjuster(L)
        _lib = L
        return L


def _declare_adjuster(L: C.CDLL) -> None:
    """Declares the bundle-adjuster entry points when the library has them."""
    fns = {
        "gbba_create": ([], C.c_void_p),
        "gbba_destroy": ([C.c_void_p], None),
    }
    for name, (args, res) in fns.items():
        f = getattr(L, name, None)
        if f is None:
            continue
        f.argtypes = args
        f.restype = res


def check(status: int) -> None:
    if status != GBBA_OK:
        msg = lib().gbba_last_error().decode("utf-8", "replace")
        if status == GBBA_ERR_OUT_OF_RANGE:
            raise IndexError(msg)
        raise GbbaError(status, msg)
