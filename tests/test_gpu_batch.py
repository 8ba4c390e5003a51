"""Batched local bundle adjustment (gbba_batch_*) against the FP64 oracle and
the single-problem GPU solver, on uneven problems mixing Brown, fisheye and
spherical cameras with fixed intrinsics (as the reference's local bundle)."""
import numpy as np
import pytest

from oracle import oracle
from opensfm_gb300 import synthetic as syn
from opensfm_gb300.pybundle import BundleBatch, adjuster_from_scene

pytestmark = pytest.mark.gpu

LOSS = ("HuberLoss", 2.0)


def _problems(n=6, seed=3):
    return syn.local_ba_problems(n, seed=seed, shots=(5, 16), points=(300, 1500), observations=(2_000, 8_000))


def _adjusters(scenes, precision="mixed"):
    return [adjuster_from_scene(s, precision=precision, loss=LOSS, irls="none", gps=False, constant_cameras=True,
                                max_iterations=100) for s in scenes]


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_batch_matches_oracle(precision):
    scenes = _problems()
    bas = _adjusters(scenes, precision)
    batch = BundleBatch()
    for ba in bas:
        batch.add(ba)
    batch.set_options(precision=precision, max_iterations=100, pcg_iterations=100,
                      pcg_tolerance=1e-4 if precision == "mixed" else 1e-10)
    batch.run()
    s = batch.summary()
    assert s["n_problems"] == len(scenes)
    assert s["n_converged"] == len(scenes)
    assert s["graph_nodes"] > 0
    for scene, ba in zip(scenes, bas):
        ref = oracle.solve(scene, loss=LOSS, irls="none", max_iterations=100, gps=False, constant_cameras=True)
        got = ba.summary()
        assert got["final_cost"] < got["initial_cost"]
        rel = abs(got["final_cost"] - ref["final_cost"]) / ref["final_cost"]
        # same trust-region rules as the oracle: FP64 follows its trajectory
        assert rel < (1e-6 if precision == "mixed" else 1e-12), (got["final_cost"], ref["final_cost"])
        assert got["iterations"] == ref["iterations"] or precision == "mixed"
        # the solution was written back into the adjuster
        assert np.abs(ba.get_points() - scene.points).max() > 0
        errs, _, _ = ba.projection_results()
        ref_rms = np.sqrt((ref["errors"][:, :2] ** 2).sum(1).mean())
        got_rms = np.sqrt((errs[:, :2] ** 2).sum(1).mean())
        assert abs(got_rms - ref_rms) < 1e-3 * max(ref_rms, 1e-12) + 1e-9


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_device_loop_graph_and_plain_launches_agree(precision):
    # the whole LM loop as one graph launch (device-side while node), one
    # graph launch per LM iteration, and plain launches: the same iterations
    scenes = _problems(4, seed=9)
    costs, iters = [], []
    for use_graph in (2, 1, 0):
        bas = _adjusters(scenes, precision)
        batch = BundleBatch()
        for ba in bas:
            batch.add(ba)
        batch.set_options(precision=precision, max_iterations=60, use_graph=use_graph, autotune=False,
                          pcg_tolerance=1e-10 if precision == "fp64" else 1e-3)
        batch.run()
        s = batch.summary()
        costs.append([ba.summary()["final_cost"] for ba in bas])
        iters.append(s["lm_iterations"])
        assert (s["graph_nodes"] > 0) == (use_graph > 0)
        assert s["graph_launches"] == {2: 1, 1: s["lm_iterations"], 0: 0}[use_graph]
        assert s["n_converged"] == len(scenes)
    np.testing.assert_allclose(costs[0], costs[1], rtol=1e-12 if precision == "fp64" else 1e-6)
    np.testing.assert_allclose(costs[0], costs[2], rtol=1e-12 if precision == "fp64" else 1e-6)
    assert iters[0] == iters[1] or precision == "mixed"


def test_device_loop_stops_at_the_iteration_limit():
    # a limit below what the problems need: the device-side loop ends there
    scenes = _problems(3, seed=4)
    bas = _adjusters(scenes, "fp64")
    batch = BundleBatch()
    for ba in bas:
        batch.add(ba)
    batch.set_options(precision="fp64", max_iterations=2, use_graph=2, autotune=False, pcg_tolerance=1e-10)
    batch.run()
    s = batch.summary()
    assert s["lm_iterations"] == 2 and s["graph_launches"] == 1
    assert all(ba.summary()["final_cost"] < ba.summary()["initial_cost"] for ba in bas)


def test_batch_rejects_free_intrinsics():
    scene = _problems(1)[0]
    ba = adjuster_from_scene(scene, loss=LOSS, irls="none", gps=False, constant_cameras=False)
    batch = BundleBatch()
    batch.add(ba)
    with pytest.raises(Exception, match="fixed intrinsics"):
        batch.run()


def test_batch_exact_steps_follow_the_dense_single_solver():
    # DENSE_SCHUR, the reference's choice for local bundles (ba_helpers.cc:
    # 336-337): every step exact (FP64, PCG to 1e-10, the iteration cap
    # raised to the camera-side unknowns) although the options ask for mixed
    # precision, 10 PCG iterations and a 1e-3 tolerance
    scenes = _problems(n=5, seed=9)
    bas = _adjusters(scenes, "mixed")
    batch = BundleBatch()
    for ba in bas:
        batch.add(ba)
    batch.set_options(precision="mixed", max_iterations=100, pcg_iterations=10, pcg_tolerance=1e-3)
    batch.set_linear_solver_type("DENSE_SCHUR")
    batch.run()
    assert batch.summary()["n_converged"] == len(scenes)
    for scene, ba in zip(scenes, bas):
        single = adjuster_from_scene(scene, precision="fp64", loss=LOSS, irls="none", gps=False,
                                     constant_cameras=True, max_iterations=100, linear_solver="DENSE_SCHUR")
        single.run()
        ref = single.summary()
        got = ba.summary()
        assert "DENSE_SCHUR" in ba.full_report()
        rel = abs(got["final_cost"] - ref["final_cost"]) / ref["final_cost"]
        assert rel < 1e-10, (got["final_cost"], ref["final_cost"])
        assert got["iterations"] == ref["iterations"]

