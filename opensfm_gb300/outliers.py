"""Post-solve outlier selection on the device: the observation test of
sfm::BAHelpers::RemoveOutliers (opensfm/src/lib/sfm/src/ba_helpers.cc:
1847-1975), binding ``gbba_find_outliers`` / ``gbba_adjuster_find_outliers``
(include/gbba.h).  No CPU fallback."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib


class OutlierConfig(C.Structure):
    _fields_ = [("filter_type", C.c_int), ("fixed_threshold", C.c_double), ("auto_ratio", C.c_double),
                ("weight_threshold", C.c_double)]


class OutlierResult(C.Structure):
    _fields_ = [("threshold", C.c_double), ("n_outliers", C.c_int64), ("n_removed_points", C.c_int64),
                ("device_seconds", C.c_double)]


_FILTERS = {"FIXED": 0, "AUTO": 1}


def _L():
    L = _lib.lib()
    if not getattr(L, "_outliers_declared", False):
        D = C.POINTER(C.c_double)
        U8 = C.POINTER(C.c_uint8)
        L.gbba_find_outliers.argtypes = [D, C.c_int, D, C.POINTER(C.c_int32), C.c_int64, C.c_int64,
                                         C.POINTER(OutlierConfig), U8, U8, C.POINTER(OutlierResult)]
        L.gbba_adjuster_find_outliers.argtypes = [C.c_void_p, C.POINTER(OutlierConfig), U8, U8,
                                                  C.POINTER(OutlierResult)]
        L._outliers_declared = True
    return L


def config(filter_type: str = "FIXED", fixed_threshold: float = 0.006, auto_ratio: float = 3.0,
           weight_threshold: float = 0.5) -> OutlierConfig:
    """The reference's configuration keys bundle_outlier_filtering_type,
    bundle_outlier_fixed_threshold, bundle_outlier_auto_ratio and
    bundle_outlier_weight_threshold (defaults as in opensfm/config.py)."""
    return OutlierConfig(_FILTERS[filter_type], fixed_threshold, auto_ratio, weight_threshold)


def find_outliers(errors, weights, obs_point, n_points: int, stats: dict | None = None, **cfg):
    """Returns (threshold, outlier flags [n], removed-point flags [n_points]).
    ``stats``, when given, receives the counts and the device time."""
    e = np.ascontiguousarray(errors, dtype=np.float64)
    w = np.ascontiguousarray(weights, dtype=np.float64)
    p = np.ascontiguousarray(obs_point, dtype=np.int32)
    n = len(w)
    if e.ndim != 2 or e.shape[0] != n or e.shape[1] < 2 or p.shape != (n,):
        raise ValueError("find_outliers: errors [n, >=2], weights [n] and obs_point [n] expected")
    flags = np.zeros(n, np.uint8)
    removed = np.zeros(max(1, n_points), np.uint8)
    res = OutlierResult()
    c = config(**cfg)
    D = C.POINTER(C.c_double)
    U8 = C.POINTER(C.c_uint8)
    _lib.check(_L().gbba_find_outliers(e.ctypes.data_as(D), e.shape[1], w.ctypes.data_as(D),
                                       p.ctypes.data_as(C.POINTER(C.c_int32)), n, n_points, C.byref(c),
                                       flags.ctypes.data_as(U8), removed.ctypes.data_as(U8), C.byref(res)))
    if stats is not None:
        stats.update(n_outliers=int(res.n_outliers), n_removed_points=int(res.n_removed_points),
                     device_seconds=float(res.device_seconds))
    return res.threshold, flags.astype(bool), removed[:n_points].astype(bool)


def adjuster_outliers(ba, **cfg):
    """The same on a BundleAdjuster's last solve; observations and points in
    insertion order.  Returns (threshold, outlier flags, removed-point flags)."""
    L = _L()
    n = int(L.gbba_num_projections(ba._h))
    n_points = int(L.gbba_num_points(ba._h))
    flags = np.zeros(max(1, n), np.uint8)
    removed = np.zeros(max(1, n_points), np.uint8)
    res = OutlierResult()
    c = config(**cfg)
    U8 = C.POINTER(C.c_uint8)
    _lib.check(L.gbba_adjuster_find_outliers(ba._h, C.byref(c), flags.ctypes.data_as(U8),
                                             removed.ctypes.data_as(U8), C.byref(res)))
    return res.threshold, flags[:n].astype(bool), removed[:n_points].astype(bool)


__all__ = ["OutlierConfig", "config", "find_outliers", "adjuster_outliers"]
