"""GPU residual + Jacobian evaluation against the FP64 oracle.

FP64 device path: element-wise within 1e-10 of the block's magnitude
(different but equivalent operation order: the device precomputes the
per-shot rotation derivative and folds the affine stage).
Mixed path (FP32 arithmetic on camera-centred coordinates): within 2e-4 of
the block's magnitude, and residuals within 1e-3 px.
"""
import numpy as np
import pytest

from oracle import oracle
from opensfm_gb300 import _lib
from opensfm_gb300 import synthetic as syn
from opensfm_gb300.scene import (BROWN, DUAL, FISHEYE, FISHEYE62, FISHEYE624, FISHEYE_OPENCV,
                                 PERSPECTIVE, RADIAL, SIMPLE_RADIAL, SPHERICAL, Evaluator,
                                 evaluate_projections)

pytestmark = pytest.mark.gpu

ALL_MODELS = [PERSPECTIVE, BROWN, FISHEYE, FISHEYE_OPENCV, FISHEYE62, FISHEYE624, DUAL, RADIAL,
              SIMPLE_RADIAL]


def _compare(scene, got, rel):
    ref = oracle.evaluate_scene(scene)
    names = ["residuals", "jac_camera", "jac_instance", "jac_rig_camera", "jac_point"]
    for name, r in zip(names, ref):
        g = getattr(got, name)
        assert g.shape == r.shape, name
        scale = max(1.0, float(np.abs(r).max()))
        err = float(np.abs(g - r).max())
        assert err <= rel * scale, f"{name}: max err {err:g} vs scale {scale:g}"


@pytest.mark.parametrize("model", ALL_MODELS)
def test_single_model_fp64(model):
    scene = syn.random_scene(11 + model, [model], n_shots=10, n_points=200)
    _compare(scene, evaluate_projections(scene, _lib.PRECISION_FP64), 1e-10)


@pytest.mark.parametrize("model", ALL_MODELS)
def test_single_model_mixed(model):
    scene = syn.random_scene(31 + model, [model], n_shots=10, n_points=200)
    _compare(scene, evaluate_projections(scene, _lib.PRECISION_MIXED), 2e-4)


@pytest.mark.parametrize("precision,tol", [(_lib.PRECISION_FP64, 1e-10), (_lib.PRECISION_MIXED, 2e-4)])
def test_mixed_models_with_spherical_and_rig(precision, tol):
    scene = syn.random_scene(5, [BROWN, FISHEYE, SPHERICAL, FISHEYE624], n_shots=12, n_points=150,
                             rig=True)
    assert scene.layout() == (3, 16)
    _compare(scene, evaluate_projections(scene, precision), tol)


def test_rig_without_spherical_fp64():
    scene = syn.random_scene(9, [PERSPECTIVE, BROWN], rig=True)
    _compare(scene, evaluate_projections(scene, _lib.PRECISION_FP64), 1e-10)


@pytest.mark.parametrize("precision,tol", [(_lib.PRECISION_FP64, 1e-10), (_lib.PRECISION_MIXED, 2e-4)])
def test_rig_partly_applied(precision, tol):
    # some shots have no rig camera, others an unused one: their rig-camera
    # block is zero (projection_errors.h:184-188) while rig shots keep theirs
    scene = syn.random_scene(13, [PERSPECTIVE, BROWN], n_shots=12, rig=True)
    scene.shot_rig_camera[::3] = -1
    scene.rig_camera_used[1] = 0
    got = evaluate_projections(scene, precision)
    _compare(scene, got, tol)
    no_rig = (scene.shot_rig_camera[scene.obs_shot] < 0) | (scene.rig_camera_used[scene.shot_rig_camera[scene.obs_shot]] == 0)
    assert no_rig.any() and (~no_rig).any()
    assert np.all(got.jac_rig_camera[no_rig] == 0)
    assert np.abs(got.jac_rig_camera[~no_rig]).max() > 0


def test_utm_offsets_mixed_precision():
    """Georeferenced scene (x ~ 5e5, y ~ 4e6): the mixed path centres in FP64
    before the FP32 cast, so residuals stay within 1e-3 px."""
    scene = syn.aerial_scene(seed=1, nx=6, ny=6, n_points=3000)
    ref = oracle.evaluate_scene(scene)[0]
    got = evaluate_projections(scene, _lib.PRECISION_MIXED).residuals
    # residuals are in units of the observation std (1 px)
    assert np.abs(got - ref).max() < 1e-3


def test_device_resident_evaluator_repeats():
    scene = syn.ring_scene(n_points=500)
    ev = Evaluator(scene, _lib.PRECISION_MIXED)
    ev.run()
    a = ev.download()
    ev.run()
    b = ev.download()
    np.testing.assert_array_equal(a.residuals, b.residuals)
    assert ev.launches_per_run == 2
    ev.close()


def test_empty_scene():
    scene = syn.ring_scene(n_points=10)
    empty = scene.subset_observations(np.array([], np.int64))
    out = evaluate_projections(empty, _lib.PRECISION_FP64)
    assert out.residuals.shape == (0, 2)


def test_invalid_inputs_raise():
    scene = syn.ring_scene(n_points=10)
    scene.obs_point[3] = 10_000
    with pytest.raises(IndexError):
        evaluate_projections(scene, _lib.PRECISION_FP64)
    scene = syn.ring_scene(n_points=10)
    scene.obs_std[0] = 0.0
    with pytest.raises(_lib.GbbaError):
        evaluate_projections(scene, _lib.PRECISION_FP64)
