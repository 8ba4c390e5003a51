"""The differentiable projection operator (opensfm_gb300.autograd).

Checked against
  - FP64 central finite differences (torch.autograd.gradcheck);
  - the oracle's forward-mode dual-number Jacobians (the stand-in for the
    reference's Ceres autodiff Jacobians, reprojection_errors_test.cc),
    contracted with a random residual gradient;
  - the FP64 evaluator's residuals;
and stored-Jacobian vs recompute (matrix-free) backward, FP32 vs FP64.
"""
import numpy as np
import pytest

from oracle import oracle
from opensfm_gb300 import _lib
from opensfm_gb300 import synthetic as syn
from opensfm_gb300.scene import BROWN, FISHEYE62, PERSPECTIVE, evaluate_projections

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _ops():
    from opensfm_gb300 import autograd as ag
    return ag


def _scene(model, seed, n_shots=6, n_points=40, obs_per_point=3):
    return syn.random_scene(seed, [model], n_shots=n_shots, n_points=n_points, obs_per_point=obs_per_point)


@pytest.mark.parametrize("model", [BROWN, FISHEYE62])
def test_gradcheck_fp64_finite_differences(model):
    ag = _ops()
    scene = _scene(model, 3, n_shots=4, n_points=12, obs_per_point=2)
    cams, poses, pts, obs = ag.observations_from_scene(scene)
    for recompute in (False, True):
        inputs = tuple(t.clone().requires_grad_(True) for t in (cams, poses, pts))
        assert torch.autograd.gradcheck(lambda c, p, x: ag.project_residuals(c, p, x, obs, recompute), inputs,
                                        eps=1e-6, atol=1e-5, rtol=1e-4)


@pytest.mark.parametrize("model", [BROWN, FISHEYE62, PERSPECTIVE])
def test_backward_matches_oracle_dual_number_jacobians(model):
    ag = _ops()
    scene = _scene(model, 7)
    cams, poses, pts, obs = ag.observations_from_scene(scene)
    cams.requires_grad_(True), poses.requires_grad_(True), pts.requires_grad_(True)
    res = ag.project_residuals(cams, poses, pts, obs)
    g = torch.randn_like(res)
    res.backward(g)
    gh = g.cpu().numpy()
    C = oracle.num_params(model)
    want_c = np.zeros((len(scene.camera_values), 16))
    want_p = np.zeros((len(scene.rig_instance_poses), 6))
    want_x = np.zeros((len(scene.points), 3))
    want_r = np.zeros((scene.n_observations, 2))
    for i in range(scene.n_observations):
        sh, pt = scene.obs_shot[i], scene.obs_point[i]
        cam, inst = scene.shot_camera[sh], scene.shot_rig_instance[sh]
        r, jc, ji, _, jp = oracle.residual_jacobian(model, scene.camera_values[cam][:C], scene.rig_instance_poses[inst],
                                                    None, scene.points[pt], scene.obs_xy[i], scene.obs_std[i], ad=True)
        want_r[i] = r
        want_c[cam, :C] += jc.T @ gh[i]
        want_p[inst] += ji.T @ gh[i]
        want_x[pt] += jp.T @ gh[i]
    np.testing.assert_allclose(res.detach().cpu().numpy(), want_r, rtol=0, atol=1e-9 * np.abs(want_r).max())
    for got, want in ((cams.grad, want_c), (poses.grad, want_p), (pts.grad, want_x)):
        np.testing.assert_allclose(got.cpu().numpy(), want, rtol=0, atol=1e-9 * max(1.0, np.abs(want).max()))


def test_forward_matches_evaluator_and_modes_agree():
    ag = _ops()
    scene = syn.random_scene(11, [BROWN], n_shots=10, n_points=400, obs_per_point=5)
    ref = evaluate_projections(scene, _lib.PRECISION_FP64).residuals
    out = {}
    for dtype in (torch.float64, torch.float32):
        for recompute in (False, True):
            cams, poses, pts, obs = ag.observations_from_scene(scene, dtype=dtype)
            leaves = [t.requires_grad_(True) for t in (cams, poses, pts)]
            res = ag.project_residuals(*leaves, obs, recompute)
            (res * res).sum().backward()
            out[(dtype, recompute)] = (res.detach().double().cpu().numpy(),
                                       [t.grad.double().cpu().numpy() for t in leaves])
    np.testing.assert_allclose(out[(torch.float64, False)][0], ref, rtol=0, atol=1e-10 * np.abs(ref).max())
    for dtype, tol in ((torch.float64, 1e-12), (torch.float32, 1e-5)):
        (r0, g0), (r1, g1) = out[(dtype, False)], out[(dtype, True)]
        np.testing.assert_allclose(r0, r1, rtol=0, atol=tol * np.abs(r0).max())
        for a, b in zip(g0, g1):
            np.testing.assert_allclose(a, b, rtol=0, atol=tol * 10 * max(1.0, np.abs(a).max()))
    # FP32 against FP64 (residuals ~1e3 sigma: FP32 relative precision)
    r64, g64 = out[(torch.float64, True)]
    r32, g32 = out[(torch.float32, True)]
    assert np.abs(r32 - r64).max() < 1e-3 * max(1.0, np.abs(r64).max())
    for a, b in zip(g32, g64):
        assert np.abs(a - b).max() < 1e-3 * max(1.0, np.abs(b).max())


def test_bad_indices_raise():
    ag = _ops()
    scene = _scene(BROWN, 5)
    scene.obs_point[3] = len(scene.points)
    cams, poses, pts, obs = ag.observations_from_scene(scene)
    with pytest.raises(IndexError, match="observation 3"):
        ag.project_residuals(cams, poses, pts, obs)
