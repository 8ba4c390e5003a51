"""gbba_evaluate_projections_noalloc against gbba_evaluate_projections and
the FP64 oracle.

The no-allocation entry point evaluates a scene held in caller-owned device
memory into caller-owned device outputs.  Two calls in a row must both agree
with the host-buffer entry point (FP64) on the same scene, and with the FP64
oracle within the FP64 evaluation bar (1e-10 of each block's magnitude); bad
inputs must come back as the same status codes.  This file is collected last
so that it also runs after every other test in one process.
"""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle
from opensfm_gb300 import _lib
from opensfm_gb300 import synthetic as syn
from opensfm_gb300.scene import BROWN, FISHEYE, FISHEYE624, PERSPECTIVE, SPHERICAL, evaluate_projections

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

NAMES = ["residuals", "jac_camera", "jac_instance", "jac_rig_camera", "jac_point"]


def _fn():
    L = _lib.lib()
    f = L.gbba_evaluate_projections_noalloc
    f.argtypes = [C.POINTER(_lib.Scene), C.c_int, C.c_int, C.POINTER(_lib.EvalOutput), C.c_void_p]
    f.restype = C.c_int
    return f


class DeviceScene:
    """The scene's arrays copied to cuda:0 by the caller (torch owns them)."""

    def __init__(self, scene):
        _ctypes_map()
        dev = torch.device("cuda:0")
        self.t = {}

        def put(name, a):
            t = torch.from_numpy(np.ascontiguousarray(a)).to(dev)
            self.t[name] = t
            return C.cast(C.c_void_p(t.data_ptr()), C.POINTER(_CT[t.dtype]))

        s = _lib.Scene()
        s.n_cameras = len(scene.camera_projection)
        s.camera_projection = put("cp", scene.camera_projection)
        s.camera_values = put("cv", scene.camera_values)
        s.n_rig_instances = len(scene.rig_instance_poses)
        s.rig_instance_poses = put("ip", scene.rig_instance_poses)
        s.n_rig_cameras = len(scene.rig_camera_poses)
        if s.n_rig_cameras:
            s.rig_camera_poses = put("rp", scene.rig_camera_poses)
            s.rig_camera_used = put("ru", scene.rig_camera_used)
        s.n_shots = len(scene.shot_camera)
        s.shot_rig_instance = put("si", scene.shot_rig_instance)
        s.shot_rig_camera = put("sr", scene.shot_rig_camera)
        s.shot_camera = put("sc", scene.shot_camera)
        s.n_points = len(scene.points)
        s.points = put("pt", scene.points)
        s.n_observations = len(scene.obs_shot)
        s.obs_shot = put("os", scene.obs_shot)
        s.obs_point = put("op", scene.obs_point)
        s.obs_xy = put("ox", scene.obs_xy)
        s.obs_std = put("sd", scene.obs_std)
        self.s = s


_CT = {}


def _ctypes_map():
    _CT.update({torch.float64: C.c_double, torch.int32: C.c_int32, torch.uint8: C.c_uint8})


class DeviceOutputs:
    def __init__(self, n, nr, cmax):
        shapes = [(n, nr), (n, nr, cmax), (n, nr, 6), (n, nr, 6), (n, nr, 3)]
        # filled with NaN so that an unwritten element cannot pass
        self.t = [torch.full(sh, float("nan"), dtype=torch.float64, device="cuda:0") for sh in shapes]
        o = _lib.EvalOutput()
        for name, t in zip(NAMES, self.t):
            setattr(o, name, C.cast(C.c_void_p(t.data_ptr()), C.POINTER(C.c_double)))
        self.o = o

    def host(self):
        torch.cuda.synchronize()
        return [t.cpu().numpy() for t in self.t]


def _call(dscene, nr, cmax, outs):
    stream = torch.cuda.current_stream().cuda_stream
    return _fn()(C.byref(dscene.s), nr, cmax, C.byref(outs.o), C.c_void_p(stream))


SCENES = [
    ("perspective", lambda: syn.random_scene(3, [PERSPECTIVE], n_shots=10, n_points=300)),
    ("mixed_models_spherical_rig",
     lambda: syn.random_scene(5, [BROWN, FISHEYE, SPHERICAL, FISHEYE624], n_shots=12, n_points=150, rig=True)),
    ("aerial_utm", lambda: syn.aerial_scene(seed=1, nx=6, ny=6, n_points=2000)),
]


@pytest.mark.parametrize("name,make", SCENES, ids=[s[0] for s in SCENES])
def test_noalloc_matches_evaluate_projections_twice(name, make):
    scene = make()
    nr, cmax = scene.layout()
    ref = evaluate_projections(scene, _lib.PRECISION_FP64)
    orc = oracle.evaluate_scene(scene)
    dscene = DeviceScene(scene)
    got = []
    for _ in range(2):
        outs = DeviceOutputs(scene.n_observations, nr, cmax)
        _lib.check(_call(dscene, nr, cmax, outs))
        got.append(outs.host())
    for call in got:
        for k, nm in enumerate(NAMES):
            r = getattr(ref, nm)
            g = call[k]
            assert g.shape == r.shape, nm
            assert np.isfinite(g).all(), nm
            scale = max(1.0, float(np.abs(r).max()))
            err = float(np.abs(g - r).max())
            # same FP64 arithmetic; the single-model specialisation of the
            # host-buffer path may contract a few operations differently
            assert err <= 1e-12 * scale, f"{name} {nm}: {err:g} (scale {scale:g})"
            # and the oracle (same bar as the FP64 evaluation tests)
            o = orc[k]
            oscale = max(1.0, float(np.abs(o).max()))
            oerr = float(np.abs(g - o).max())
            assert oerr <= 1e-10 * oscale, f"{name} {nm} vs oracle: {oerr:g} (scale {oscale:g})"
    for k in range(5):
        np.testing.assert_array_equal(got[0][k], got[1][k])


def test_noalloc_rejects_bad_inputs():
    scene = syn.random_scene(3, [PERSPECTIVE], n_shots=10, n_points=300)
    nr, cmax = scene.layout()
    n = scene.n_observations
    # an observation of a missing point: found on the device, reported as
    # the out-of-range status, nothing read out of bounds
    bad = syn.random_scene(3, [PERSPECTIVE], n_shots=10, n_points=300)
    bad.obs_point[7] = 300
    d = DeviceScene(bad)
    outs = DeviceOutputs(n, nr, cmax)
    assert _call(d, nr, cmax, outs) == _lib.GBBA_ERR_OUT_OF_RANGE
    assert b"observation 7" in _lib.lib().gbba_last_error()
    # non-positive std deviation
    bad = syn.random_scene(3, [PERSPECTIVE], n_shots=10, n_points=300)
    bad.obs_std[11] = 0.0
    d = DeviceScene(bad)
    assert _call(d, nr, cmax, outs) == _lib.GBBA_ERR_INVALID_ARGUMENT
    # output narrower than the camera needs
    d = DeviceScene(syn.random_scene(4, [BROWN], n_shots=10, n_points=100))
    outs3 = DeviceOutputs(d.s.n_observations, 2, 3)
    assert _call(d, 2, 3, outs3) == _lib.GBBA_ERR_INVALID_ARGUMENT
    # host memory is refused before any kernel runs
    host = scene.ctypes()
    st = _fn()(C.byref(host), nr, cmax, C.byref(outs.o), None)
    assert st == _lib.GBBA_ERR_INVALID_ARGUMENT
    assert b"not device memory" in _lib.lib().gbba_last_error()
    # more shots than the fixed scratch holds
    d = DeviceScene(scene)
    d.s.n_shots = 8193
    assert _call(d, nr, cmax, outs) == _lib.GBBA_ERR_INVALID_ARGUMENT
    assert b"at most 8192" in _lib.lib().gbba_last_error()
    # a shot whose camera does not exist: found by the shot kernel, reported
    # with the shot's index
    bad = syn.random_scene(3, [PERSPECTIVE], n_shots=10, n_points=300)
    bad.shot_camera[4] = 5
    d = DeviceScene(bad)
    assert _call(d, nr, cmax, outs) == _lib.GBBA_ERR_OUT_OF_RANGE
    assert b"shot 4" in _lib.lib().gbba_last_error()
    # an unknown projection type
    bad = syn.random_scene(3, [PERSPECTIVE], n_shots=10, n_points=300)
    bad.camera_projection[0] = 42
    d = DeviceScene(bad)
    assert _call(d, nr, cmax, outs) == _lib.GBBA_ERR_RUNTIME
    assert b"ProjectionType" in _lib.lib().gbba_last_error()
    # a good call afterwards still matches
    good = DeviceScene(scene)
    outs = DeviceOutputs(n, nr, cmax)
    _lib.check(_call(good, nr, cmax, outs))
    ref = evaluate_projections(scene, _lib.PRECISION_FP64)
    np.testing.assert_allclose(outs.host()[0], ref.residuals, rtol=0, atol=1e-12 * max(1, np.abs(ref.residuals).max()))


def test_noalloc_null_outputs_are_skipped():
    """Outputs passed as NULL are not written; the others match the full call."""
    scene = syn.random_scene(5, [BROWN, FISHEYE, SPHERICAL, FISHEYE624], n_shots=12, n_points=150, rig=True)
    nr, cmax = scene.layout()
    d = DeviceScene(scene)
    full = DeviceOutputs(scene.n_observations, nr, cmax)
    _lib.check(_call(d, nr, cmax, full))
    part = DeviceOutputs(scene.n_observations, nr, cmax)
    part.o.jac_camera = C.POINTER(C.c_double)()
    part.o.jac_rig_camera = C.POINTER(C.c_double)()
    _lib.check(_call(d, nr, cmax, part))
    a, b = full.host(), part.host()
    for k in (0, 2, 4):
        np.testing.assert_array_equal(a[k], b[k])
    for k in (1, 3):
        assert np.isnan(b[k]).all()
