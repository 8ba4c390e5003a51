"""Shared pytest configuration.

Tests marked ``gpu`` need a CUDA device and the built ``libgbba.so``; the
rest run on any machine (they build and load the oracle and check the C ABI
exports without launching kernels).
"""
import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the compiled extension")
    config.addinivalue_line("markers", "slow: long-running case")


@pytest.fixture(scope="session", autouse=True)
def _built():
    from opensfm_gb300.build import build_all
    build_all()
    yield


def _has_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:  # pragma: no cover
        return False


# Dependency order of the GPU files: the solver and its kernels first, then
# the constraint terms built on the solver, then the callers built on both
# (local bundles).  Under -x a failure in a caller then cannot hide the
# result of the layer it stands on.  Files not listed keep their place
# after these.
_GPU_ORDER = ("test_gpu_evaluate.py", "test_gpu_solver.py", "test_gpu_dense.py", "test_gpu_matrix_free.py",
              "test_gpu_batch.py", "test_gpu_autograd.py", "test_gpu_outliers.py", "test_gpu_covariance.py",
              "test_gpu_orientation.py", "test_gpu_relative.py", "test_gpu_relative_motion.py",
              "test_gpu_position_std.py", "test_gpu_depth.py", "test_gpu_bias.py", "test_gpu_ba_helpers.py", "test_gpu_ba_full.py")


def _file_rank(item) -> int:
    name = Path(str(item.fspath)).name
    return _GPU_ORDER.index(name) if name in _GPU_ORDER else len(_GPU_ORDER)


def pytest_collection_modifyitems(config, items):
    items.sort(key=_file_rank)  # stable: the order within a file stays
    if _has_gpu():
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)
