"""Two-level PCG preconditioner on the GPU (coarse_space.h): block-Jacobi
plus a coarse space of cluster similarity modes.  The preconditioner changes
how fast PCG converges, not the problem: solves with and without it reach
the oracle's optimum, and with it PCG takes fewer iterations."""
import numpy as np
import pytest

from oracle import oracle
from opensfm_gb300 import synthetic as syn
from opensfm_gb300.pybundle import adjuster_from_scene

pytestmark = pytest.mark.gpu


def _solve(scene, precision, leaf, **kw):
    ba = adjuster_from_scene(scene, precision=precision, loss=("HuberLoss", 2.0), irls="none", gps=True,
                             linear_solver="ITERATIVE_SCHUR", coarse_leaf=leaf, **kw)
    ba.run()
    return ba


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_aerial_two_level_matches_oracle_in_fewer_iterations(precision):
    # tight PCG tolerances (mixed: FP64 iterative refinement) make every
    # linear solve long enough for the probes to pay, so the coarse space is
    # probed from the second linearization on
    scene = syn.aerial_scene(seed=2, nx=16, ny=16, n_points=12000)
    ref = oracle.solve(scene, loss=("HuberLoss", 2.0), irls="none", max_iterations=60, gps=True)
    tol = 1e-10 if precision == "fp64" else 1e-8
    runs = {}
    for leaf in (0, 8):
        ba = _solve(scene, precision, leaf, max_iterations=60, pcg_tolerance=tol)
        s = ba.summary()
        rel = abs(s["final_cost"] - ref["final_cost"]) / ref["final_cost"]
        assert rel < (1e-9 if precision == "fp64" else 1e-7), (leaf, s["final_cost"], ref["final_cost"])
        runs[leaf] = (ba.trace(), ba.coarse_info())
    plain, two = runs[0][0], runs[8][0]
    assert runs[0][1]["probes"] == 0
    info = runs[8][1]
    assert info["clusters"] == 32 and info["colours"] >= 2
    assert info["probes"] > 0 and info["probes"] % (7 * info["colours"]) == 0  # 7 per colour and probed linearization
    # the first linear solve is block-Jacobi in both (mixed-precision counts
    # vary by a few iterations from run to run); then PCG iterations drop
    assert abs(two[1, 4] - plain[1, 4]) <= 0.05 * plain[1, 4]
    assert two[2:, 4].sum() < 0.5 * plain[2:, 4].sum(), (two[:, 4], plain[:, 4])


def test_two_level_graph_and_host_loop_agree():
    # the coarse correction inside the PCG graph and launched kernel by
    # kernel: the same FP64 trajectory (the coarse sums run in a fixed order)
    scene = syn.aerial_scene(seed=6, nx=10, ny=10, n_points=5000)
    traces = []
    for graph in (True, False):
        ba = _solve(scene, "fp64", 6, max_iterations=8, pcg_tolerance=1e-10, pcg_graph=graph)
        assert ba.coarse_info()["probes"] > 0
        traces.append(ba.trace())
    a, b = traces
    assert a.shape == b.shape
    np.testing.assert_allclose(a[:, 1], b[:, 1], rtol=1e-8)  # FP64 atomics of the passes, as for block-Jacobi
    np.testing.assert_array_equal(a[:, 3], b[:, 3])
    # the iteration counts at the 1e-10 tolerance may differ by a few: the
    # coarse correction goes through the FP32 factor, whose input rounds the
    # last bits of the residual that the FP64 atomics of the passes order


def test_two_level_matrix_free_and_refinement():
    # matrix-free probes (records evaluated in every pass) and the mixed
    # path's FP64 iterative refinement (tight tolerance) run the coarse
    # correction too, and reach the stored-record FP64 solve's optimum
    scene = syn.aerial_scene(seed=4, nx=12, ny=12, n_points=6000)
    ref = _solve(scene, "fp64", 0, max_iterations=40, pcg_tolerance=1e-10).summary()["final_cost"]
    for kw in ({"precision": "fp64", "matrix_free": 1, "pcg_tolerance": 1e-10},
               {"precision": "mixed", "pcg_tolerance": 1e-8}):
        ba = _solve(scene, kw.pop("precision"), 8, max_iterations=40, **kw)
        s = ba.summary()
        assert ba.coarse_info()["probes"] > 0
        assert abs(s["final_cost"] - ref) / ref < 1e-8, (kw, s["final_cost"], ref)
