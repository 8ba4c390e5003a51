"""Dense symmetric positive definite solver of the reduced camera system.

Bindings of ``gbba_dense_spd_solve`` and ``gbba_dense_gemm_nt``
(include/gbba.h): the linear solver the bundle adjuster uses in dense mode
(the counterpart of Ceres' DENSE_SCHUR / SPARSE_SCHUR Cholesky factorization
of the reduced camera system, opensfm/src/lib/bundle/src/bundle_adjuster.cc:
1159-1190), exposed for callers that form such systems themselves.  The
factorization runs on the tensor cores; FP64 conjugate gradients
preconditioned by it give the solution FP64 accuracy.  There is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib


class _Stats(C.Structure):
    _fields_ = [("status", C.c_int), ("refinements", C.c_int), ("rel_residual", C.c_double),
                ("factor_seconds", C.c_double), ("solve_seconds", C.c_double)]


@dataclass
class DenseStats:
    status: int            # 0 solved, 1 not positive definite, 2 device wait timed out, 3 not converged
    refinements: int       # FP64 conjugate-gradient iterations
    rel_residual: float    # |D (b - A x)| / |D b|, D = diag(a)^-1/2
    factor_seconds: float
    solve_seconds: float


def _L():
    L = _lib.lib()
    if not getattr(L, "_dense_declared", False):
        D = C.POINTER(C.c_double)
        F = C.POINTER(C.c_float)
        L.gbba_dense_spd_solve.argtypes = [D, C.c_int, D, D, C.c_double, C.c_int, C.POINTER(_Stats)]
        L.gbba_dense_gemm_nt.argtypes = [F, F, F, C.c_int, C.c_int, C.c_int]
        L._dense_declared = True
    return L


def spd_solve(a: np.ndarray, b: np.ndarray, tol: float = 1e-12, max_refinements: int = 50):
    """Solves a x = b for a symmetric positive definite ``a`` (its lower
    triangle is read).  Returns ``(x, DenseStats)``."""
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    n = a.shape[0]
    if a.shape != (n, n) or b.shape != (n,):
        raise ValueError("spd_solve: a must be n x n and b of length n")
    x = np.zeros(n)
    st = _Stats()
    D = C.POINTER(C.c_double)
    _lib.check(_L().gbba_dense_spd_solve(a.ctypes.data_as(D), n, b.ctypes.data_as(D), x.ctypes.data_as(D),
                                         tol, max_refinements, C.byref(st)))
    return x, DenseStats(st.status, st.refinements, st.rel_residual, st.factor_seconds, st.solve_seconds)


def gemm_nt(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """C = a b^T on the tensor cores (FP32 in and out, three TF32 products
    per term); the row counts must be multiples of 128 and the shared
    dimension a multiple of 32."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    b = np.ascontiguousarray(b, dtype=np.float32)
    m, k = a.shape
    n, k2 = b.shape
    if k != k2:
        raise ValueError("gemm_nt: inner dimensions differ")
    c = np.zeros((m, n), np.float32)
    F = C.POINTER(C.c_float)
    _lib.check(_L().gbba_dense_gemm_nt(a.ctypes.data_as(F), b.ctypes.data_as(F), c.ctypes.data_as(F), m, n, k))
    return c


__all__ = ["DenseStats", "spd_solve", "gemm_nt"]
