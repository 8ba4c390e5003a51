"""Dense reduced-camera-system solver: the tensor-core block product and the
factor + FP64 refinement solve, against numpy FP64 on the same inputs, and
the bundle adjuster's dense mode against the oracle's dense-Schur solve.

Bars: the block product (three TF32 products per term, FP32 accumulation)
within 2e-6 max(1, sqrt(k / 256)) of |A| |B|^T per entry -- a single TF32
product would miss it by about 100x; solutions to a relative residual of
1e-11; the
FP64 dense-mode solve reproduces the oracle's LM trajectory (same Cholesky
steps up to summation order) to 1e-9 relative cost per iteration.
"""
import numpy as np
import pytest

from oracle import oracle
from opensfm_gb300 import dense
from opensfm_gb300 import synthetic as syn
from opensfm_gb300.pybundle import adjuster_from_scene

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("m,n,k", [(128, 128, 32), (256, 384, 96), (512, 256, 1024), (128, 128, 4096)])
def test_gemm_nt_matches_fp64(m, n, k):
    rng = np.random.default_rng(m + n + k)
    a = rng.standard_normal((m, k)).astype(np.float32)
    b = rng.standard_normal((n, k)).astype(np.float32)
    got = dense.gemm_nt(a, b).astype(np.float64)
    ref = a.astype(np.float64) @ b.astype(np.float64).T
    scale = np.abs(a).astype(np.float64) @ np.abs(b).astype(np.float64).T
    err = np.abs(got - ref) / scale
    # FP32 accumulation: the error grows like sqrt(k) unit roundoffs
    assert err.max() < 2e-6 * max(1.0, np.sqrt(k / 256)), err.max()


def test_gemm_nt_rejects_ragged_shapes():
    from opensfm_gb300._lib import GbbaError
    with pytest.raises(GbbaError):
        dense.gemm_nt(np.zeros((100, 32), np.float32), np.zeros((128, 32), np.float32))


def _backward_error(a, x, b):
    # componentwise relative backward error (Oettli-Prager): the smallest w
    # with (a + da) x = b + db, |da| <= w |a|, |db| <= w |b|; independent of
    # the scaling of the unknowns
    return np.max(np.abs(b - a @ x) / (np.abs(a) @ np.abs(x) + np.abs(b)))


def _spd(n, seed, cond=1e4, scales=None):
    rng = np.random.default_rng(seed)
    q, _ = np.linalg.qr(rng.standard_normal((n, n)))
    ev = np.geomspace(1.0, cond, n)
    a = (q * ev) @ q.T
    if scales is not None:
        a = a * np.outer(scales, scales)
    return 0.5 * (a + a.T)


@pytest.mark.parametrize("n", [1, 5, 127, 128, 129, 300, 1000])
def test_spd_solve_reaches_fp64_accuracy(n):
    a = _spd(n, n)
    rng = np.random.default_rng(7 * n)
    b = rng.standard_normal(n)
    x, st = dense.spd_solve(a, b)
    assert st.status == 0, st
    ref = np.linalg.solve(a, b)
    rel = np.linalg.norm(b - a @ x) / np.linalg.norm(b)
    assert rel < 1e-11, (rel, st)
    assert _backward_error(a, x, b) < 1e-11
    assert np.linalg.norm(x - ref) / np.linalg.norm(ref) < 1e-9


def test_spd_solve_badly_scaled():
    # reduced camera systems mix rotations, centres and focal lengths: column
    # scales over ten orders of magnitude are removed by the Jacobi scaling
    n = 700
    scales = np.geomspace(1e-4, 1e6, n)
    np.random.default_rng(3).shuffle(scales)
    a = _spd(n, 11, cond=1e3, scales=scales)
    b = np.random.default_rng(4).standard_normal(n)
    x, st = dense.spd_solve(a, b)
    assert st.status == 0, st
    assert _backward_error(a, x, b) < 1e-11
    d = 1.0 / np.sqrt(np.diag(a))
    ref = np.linalg.solve(a, b)
    assert np.linalg.norm((x - ref) / d) / np.linalg.norm(ref / d) < 1e-9


def test_spd_solve_reads_lower_triangle_only():
    a = _spd(200, 21)
    b = np.random.default_rng(5).standard_normal(200)
    low = np.tril(a) + np.triu(np.full_like(a, 1e30), 1)
    x, st = dense.spd_solve(low, b)
    assert st.status == 0
    assert np.linalg.norm(b - a @ x) / np.linalg.norm(b) < 1e-11


def test_spd_solve_flags_indefinite():
    a = _spd(260, 5)
    a[200, 200] = -1.0
    _, st = dense.spd_solve(a, np.ones(260))
    assert st.status == 1


def _linear_solver(ba):
    line = [l for l in ba.full_report().split("\n") if "Linear solver" in l][0]
    return line.split("Linear solver", 1)[1].strip()


def _trace_costs(ba):
    tr = ba.trace()
    return tr[:, 1]


@pytest.mark.parametrize("scene_kind", ["ring", "aerial"])
def test_dense_fp64_follows_oracle_trajectory(scene_kind):
    if scene_kind == "ring":
        scene = syn.ring_scene(n_points=2000)
        kw = dict(loss=("HuberLoss", 1.0), irls="none", max_iterations=50, gps=False)
    else:
        scene = syn.aerial_scene(seed=2, nx=8, ny=8, n_points=4000)
        kw = dict(loss=("HuberLoss", 2.0), irls="none", max_iterations=60, gps=True)
    ref = oracle.solve(scene, **kw)
    ba = adjuster_from_scene(scene, precision="fp64", linear_solver="DENSE_SCHUR", **kw)
    ba.run()
    s = ba.summary()
    assert _linear_solver(ba).startswith("DENSE_SCHUR"), _linear_solver(ba)
    assert abs(s["final_cost"] - ref["final_cost"]) / ref["final_cost"] < 1e-9
    got = _trace_costs(ba)
    want = ref["trace"]
    k = min(len(got), len(want))
    assert k >= 3
    np.testing.assert_allclose(got[:k], want[:k], rtol=1e-9)
    assert s["iterations"] == ref["iterations"]


def test_dense_mixed_matches_oracle_on_street():
    # Brown intrinsics shared by all 40 shots: the case where PCG converges
    # slowly; the dense step is exact for the FP32 Jacobian
    scene = syn.street_scene(n_shots=40, n_points=3000, seed=11, outlier_ratio=0.0)
    kw = dict(loss=("SoftLOneLoss", 1.0), irls="none", max_iterations=100, gps=False)
    ref = oracle.solve(scene, **kw)
    ba = adjuster_from_scene(scene, precision="mixed", linear_solver="DENSE_SCHUR", **kw)
    ba.run()
    s = ba.summary()
    assert abs(s["final_cost"] - ref["final_cost"]) / ref["final_cost"] < 1e-7
    # FP64 point blocks keep the formed system positive definite: no step is
    # lost to a failed factorization, and the iterations are the oracle's
    assert s["iterations"] == ref["iterations"]


def test_sparse_schur_picks_dense_for_small_systems():
    scene = syn.ring_scene(n_points=300)
    ba = adjuster_from_scene(scene, precision="mixed", loss=("HuberLoss", 1.0), irls="none", max_iterations=5,
                             gps=False)
    ba.run()
    assert _linear_solver(ba).startswith("DENSE_SCHUR")
    # mixed precision is for the iterative path: exact steps take FP64 records
    assert "FP64 records" in _linear_solver(ba)
    ba2 = adjuster_from_scene(scene, precision="mixed", loss=("HuberLoss", 1.0), irls="none", max_iterations=5,
                              gps=False, linear_solver="ITERATIVE_SCHUR")
    ba2.run()
    assert _linear_solver(ba2).startswith("ITERATIVE_SCHUR")
