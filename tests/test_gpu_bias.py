"""Optimised camera biases: GPU solves against the FP64 CPU oracle.

The GPS priors of a small aerial problem carry a known similarity bias and
15 ground control points fix the frame (test_bias_host.biased_aerial).  With
every bias parameter optimised (SetCameraBias's parameters_to_optimize,
bundle_adjuster.cc:131-140), the GPU solve reaches the oracle's final cost
(within 1e-6) and bias, in FP64 and mixed precision, on the PCG and the
exact (dense) path; a subset of the parameters (the translation, as
DetermineGCPBiasParameters picks for one ground control point,
ba_helpers.cc:1804-1845) keeps the rest at its value.
"""
import numpy as np
import pytest

from oracle import oracle
from opensfm_gb300.pybundle import adjuster_from_scene
from test_bias_host import biased_aerial

pytestmark = pytest.mark.gpu


def _solve(scene, precision, solver, bias, priors):
    pcg = 1e-10 if precision == "fp64" else 1e-4
    ba = adjuster_from_scene(scene, precision=precision, loss=("HuberLoss", 2.0), irls="none", max_iterations=60,
                             gps=True, constant_cameras=True, pcg_tolerance=pcg, linear_solver=solver, bias=bias,
                             point_priors=priors)
    ba.run()
    b = ba.get_bias("0")
    return ba.summary(), np.r_[b.rotation, b.translation, b.scale]


@pytest.mark.parametrize("solver", ["ITERATIVE_SCHUR", "SPARSE_SCHUR"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_optimised_bias_matches_oracle(precision, solver):
    scene, _, priors = biased_aerial()
    bias = (np.zeros(3), np.zeros(3), 1.0, list(range(7)))
    ref = oracle.solve(scene, loss=("HuberLoss", 2.0), irls="none", max_iterations=60, gps=True,
                       constant_cameras=True, bias=bias, point_priors=priors)
    s, b = _solve(scene, precision, solver, bias, priors)
    rel = abs(s["final_cost"] - ref["final_cost"]) / ref["final_cost"]
    assert rel < 1e-6, (s["final_cost"], ref["final_cost"])
    np.testing.assert_allclose(b[:3], ref["bias"][:3], atol=1e-5)
    np.testing.assert_allclose(b[3:6], ref["bias"][3:6], atol=1e-3)
    np.testing.assert_allclose(b[6], ref["bias"][6], atol=1e-5)


def test_bias_subset_keeps_the_fixed_parameters():
    scene, _, priors = biased_aerial(seed=5)
    start = (np.array([0.01, 0.0, 0.0]), np.zeros(3), 1.01, [3, 4, 5])
    ref = oracle.solve(scene, loss=("HuberLoss", 2.0), irls="none", max_iterations=60, gps=True,
                       constant_cameras=True, bias=start, point_priors=priors)
    s, b = _solve(scene, "fp64", "SPARSE_SCHUR", start, priors)
    rel = abs(s["final_cost"] - ref["final_cost"]) / ref["final_cost"]
    assert rel < 1e-6, (s["final_cost"], ref["final_cost"])
    np.testing.assert_array_equal(b[:3], start[0])
    assert b[6] == start[2]
    np.testing.assert_allclose(b[3:6], ref["bias"][3:6], atol=1e-4)
