"""Host-side checks of the differentiable projection operator (no GPU)."""
import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from opensfm_gb300 import autograd as ag  # noqa: E402
from opensfm_gb300 import synthetic as syn  # noqa: E402
from opensfm_gb300.scene import BROWN  # noqa: E402


def _cpu_obs():
    i = lambda n: torch.zeros(n, dtype=torch.int32)  # noqa: E731
    return ag.Observations(i(1), i(2), i(2), i(4), i(4), torch.zeros(4, 2, dtype=torch.float64),
                           torch.ones(4, dtype=torch.float64), BROWN)


def test_struct_layout_matches_header():
    # gbba_device_problem_t with natural alignment on LP64
    assert ag.DeviceProblem.camera_projection.offset == 16
    assert ag.DeviceProblem.n_points.offset == 48
    assert ag.DeviceProblem.n_observations.offset == 88
    assert C.sizeof(ag.DeviceProblem) == 128
    names = [f[0] for f in ag.DeviceProblem._fields_]
    assert names[:3] == ["dtype", "model_hint", "n_cameras"] and names[-1] == "obs_std"


def test_rejects_cpu_tensors_and_mixed_dtypes():
    obs = _cpu_obs()
    cams = torch.zeros(1, 16, dtype=torch.float64)
    poses = torch.zeros(2, 6, dtype=torch.float64)
    pts = torch.zeros(3, 3, dtype=torch.float64)
    with pytest.raises(ValueError, match="CUDA"):
        ag._problem(obs, cams, poses, pts)


def test_rig_scenes_are_refused():
    scene = syn.random_scene(1, [BROWN], rig=True)
    with pytest.raises(ValueError, match="rig"):
        ag.observations_from_scene(scene, device="cpu")


def test_model_hint_from_scene():
    scene = syn.random_scene(2, [BROWN], n_shots=4, n_points=10)
    _, _, _, obs = ag.observations_from_scene(scene, device="cpu")
    assert obs.model_hint == BROWN
    mixed = syn.random_scene(2, [BROWN, 2], n_shots=4, n_points=10)
    _, _, _, obs = ag.observations_from_scene(mixed, device="cpu")
    assert obs.model_hint == -1
    assert obs.obs_shot.dtype == torch.int32 and np.array_equal(obs.obs_point.numpy(), mixed.obs_point)
