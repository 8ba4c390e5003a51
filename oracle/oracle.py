"""ctypes wrapper of the FP64 CPU oracle (test infrastructure only).

Only tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` use this module, always as the checker or the timed CPU
baseline -- never as part of the product path.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

_LIB = Path(__file__).resolve().parent / "_build" / "liboracle.so"
_lib = None

D = C.POINTER(C.c_double)


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not _LIB.exists():
            from opensfm_gb300.build import build_oracle
            build_oracle()
        L = C.CDLL(str(_LIB))
        L.oracle_num_params.argtypes = [C.c_int]
        for name in ("oracle_project", "oracle_project_ad"):
            getattr(L, name).argtypes = [C.c_int, D, D, D, D, D]
            getattr(L, name).restype = None
        for name in ("oracle_residual_jacobian", "oracle_residual_ad"):
            getattr(L, name).argtypes = [C.c_int, D, D, D, D, D, C.c_double, D, D, D, D, D]
            getattr(L, name).restype = None
        L.oracle_evaluate_scene.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, D, D, D, D, D]
        for name in ("oracle_pose_jacobian", "oracle_pose_ad"):
            getattr(L, name).argtypes = [D, D, D, D]
            getattr(L, name).restype = None
        L.oracle_loss.argtypes = [C.c_int, C.c_double, C.c_double, D]
        L.oracle_loss.restype = None
        _declare_solver(L)
        _lib = L
    return _lib


def _declare_solver(L) -> None:
    if hasattr(L, "oracle_solve"):
        L.oracle_solve.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        L.oracle_solve.restype = C.c_int


def _p(a: np.ndarray | None):
    if a is None:
        return D()
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(D)


def num_params(model: int) -> int:
    return int(lib().oracle_num_params(model))


def project(model: int, p, params, ad: bool = False):
    """(uv, J wrt camera-frame point 2x3, J wrt params 2xC)."""
    c = num_params(model)
    p = np.ascontiguousarray(p, np.float64)
    prm = np.zeros(16)
    prm[: len(params)] = params
    uv, jp, jc = np.zeros(2), np.zeros(6), np.zeros(2 * c)
    fn = lib().oracle_project_ad if ad else lib().oracle_project
    fn(model, _p(p), _p(prm), _p(uv), _p(jp), _p(jc))
    return uv, jp.reshape(2, 3), jc.reshape(2, c)


def residual_jacobian(model: int, cam, inst, rig, X, obs, std: float, ad: bool = False):
    """(r, J_camera, J_instance, J_rig_camera, J_point) of one observation."""
    c = num_params(model)
    nr = 3 if model == 6 else 2
    cam_a = np.zeros(16)
    cam_a[: len(cam)] = cam
    args = [np.ascontiguousarray(x, np.float64) for x in (inst, X, obs)]
    rig_a = None if rig is None else np.ascontiguousarray(rig, np.float64)
    r, jc, ji, jr, jp = np.zeros(nr), np.zeros(nr * c), np.zeros(nr * 6), np.zeros(nr * 6), np.zeros(nr * 3)
    fn = lib().oracle_residual_ad if ad else lib().oracle_residual_jacobian
    fn(model, _p(cam_a), _p(args[0]), _p(rig_a), _p(args[1]), _p(args[2]), std, _p(r), _p(jc), _p(ji),
       _p(jr), _p(jp))
    return r, jc.reshape(nr, c), ji.reshape(nr, 6), jr.reshape(nr, 6), jp.reshape(nr, 3)


def evaluate_scene(scene, threads: int | None = None):
    """Oracle residuals / Jacobian blocks of every observation, laid out as
    gbba_evaluate_projections returns them."""
    from opensfm_gb300.scene import alloc_outputs, output_struct  # noqa: F401
    nr, cmax = scene.layout()
    n = scene.n_observations
    res, jc, ji, jr, jp = (np.zeros((n, nr)), np.zeros((n, nr, cmax)), np.zeros((n, nr, 6)),
                           np.zeros((n, nr, 6)), np.zeros((n, nr, 3)))
    s = scene.ctypes()
    threads = threads or os.cpu_count() or 1
    lib().oracle_evaluate_scene(C.addressof(s), nr, cmax, threads, _p(res), _p(jc), _p(ji), _p(jr), _p(jp))
    return res, jc, ji, jr, jp


def pose_jacobian(X, rt, ad: bool = False):
    """(x_cam, 3x9 Jacobian [dX | d r | d t]) of PoseFunctor."""
    X = np.ascontiguousarray(X, np.float64)
    rt = np.ascontiguousarray(rt, np.float64)
    out, J = np.zeros(3), np.zeros(27)
    fn = lib().oracle_pose_ad if ad else lib().oracle_pose_jacobian
    fn(_p(X), _p(rt), _p(out), _p(J))
    return out, J.reshape(3, 9)


def loss(kind: int, threshold: float, s: float):
    rho = np.zeros(3)
    lib().oracle_loss(kind, threshold, s, _p(rho))
    return rho


def mixture_group(residuals: np.ndarray, weights: np.ndarray, density_ratio: float):
    """One mixture-reweighting group: returns (log-likelihood, new weights)."""
    r = np.ascontiguousarray(residuals, np.float64)
    w = np.array(weights, np.float64)
    f = lib().oracle_mixture_group
    f.argtypes = [C.c_int, C.c_int64, D, D, C.c_double]
    f.restype = C.c_double
    ll = f(r.shape[1], r.shape[0], _p(r), _p(w), density_ratio)
    return ll, w


# ---------------------------------------------------------------------------
# FP64 CPU bundle-adjustment solve (oracle/solver.cpp)

U8 = C.POINTER(C.c_uint8)
I32 = C.POINTER(C.c_int32)


class _Problem(C.Structure):
    _fields_ = [
        ("n_cameras", C.c_int32), ("camera_model", I32), ("camera_values", D), ("camera_prior", D),
        ("camera_sigma", D), ("camera_free", U8), ("camera_log", U8),
        ("n_instances", C.c_int32), ("instance_poses", D), ("instance_free", U8), ("instance_has_gps", U8),
        ("gps_position", D), ("gps_std", D),
        ("n_rig_cameras", C.c_int32), ("rig_poses", D), ("rig_free", U8), ("rig_used", U8), ("rig_has_prior", U8),
        ("rig_prior", D), ("rig_sigma", D),
        ("n_shots", C.c_int32), ("shot_instance", I32), ("shot_rig", I32), ("shot_camera", I32),
        ("n_points", C.c_int64), ("points", D), ("point_free", U8), ("point_has_prior", U8), ("point_prior", D),
        ("point_sigma", D), ("point_has_altitude", U8),
        ("n_obs", C.c_int64), ("obs_shot", I32), ("obs_point", I32), ("obs_xy", D), ("obs_std", D), ("obs_gcp", U8),
        ("n_orient", C.c_int32), ("orient_kind", I32), ("orient_shot", I32), ("orient_target", D), ("orient_std", D),
        ("n_rel", C.c_int32), ("rel_kind", I32), ("rel_shots", I32), ("rel_params", D), ("rel_loss", C.c_int32),
        ("rel_loss_threshold", C.c_double), ("heat_grid", D), ("heat_n", C.c_int64), ("heat_width", C.c_int32),
        ("heat_resolution", C.c_double), ("n_scales", C.c_int32), ("scales", D), ("scale_free", U8),
        ("n_depth", C.c_int64), ("depth_obs", C.POINTER(C.c_int64)), ("depth_value", D), ("depth_std", D),
        ("depth_radial", U8),
    ]


class _Options(C.Structure):
    _fields_ = [("max_iterations", C.c_int32), ("loss", C.c_int32), ("loss_threshold", C.c_double),
                ("irls", C.c_int32), ("density_ratio", C.c_double), ("skip_initial_reweighting", C.c_int32),
                ("threads", C.c_int32)]


class _Result(C.Structure):
    _fields_ = [("camera_values", D), ("instance_poses", D), ("rig_poses", D), ("points", D), ("scales", D),
                ("obs_weights", D), ("obs_errors", D), ("trace_cost", D), ("trace_capacity", C.c_int32),
                ("trace_n", C.c_int32), ("initial_cost", C.c_double), ("final_cost", C.c_double),
                ("iterations", C.c_int32), ("successful", C.c_int32), ("termination", C.c_int32)]


LOSSES = {"TrivialLoss": 0, "HuberLoss": 1, "SoftLOneLoss": 2, "CauchyLoss": 3, "ArctanLoss": 4}

# default prior standard deviation per parameter of each model (1 for the
# parameters BundleAdjuster::GetDefaultCameraSigma configures, 0 otherwise)
_SIGMA_ONE = {0: [1, 1, 1], 1: [1] * 9, 2: [1, 1, 1], 3: [1, 1, 1, 0, 1, 1, 1, 1],
              4: [1, 1, 1, 0, 0, 0, 1, 1, 1, 1, 1, 1], 5: [1, 1, 1, 0, 0, 0, 1, 1, 0, 0, 0, 0, 1, 1, 1, 1],
              6: [0], 7: [1, 1, 1, 1], 8: [1] * 6, 9: [1] * 5}
_LOG = {0: [0, 0, 1], 1: [0, 0, 0, 0, 0, 1, 1, 0, 0], 2: [0, 0, 1], 3: [0, 0, 0, 0, 1, 1, 0, 0],
        4: [0] * 8 + [1, 1, 0, 0], 5: [0] * 12 + [1, 1, 0, 0], 6: [0], 7: [0, 0, 0, 1], 8: [0, 0, 1, 1, 0, 0],
        9: [0, 1, 1, 0, 0]}


ORIENTATION_KINDS = {"up_vector": 0, "pan": 1, "tilt": 2, "roll": 3}


def orientation_residual(kind: str, target, std: float, instance_rotation, camera_rotation=None):
    """Scaled residuals and Jacobian [m][6] of one absolute orientation
    constraint (oracle/solver.cpp restatement)."""
    L = lib()
    f = L.oracle_orientation_residual
    f.argtypes = [C.c_int, D, C.c_double, D, D, D, D]
    f.restype = C.c_int
    t = np.zeros(3)
    v = np.atleast_1d(np.asarray(target, np.float64))
    t[: len(v)] = v
    ri = np.ascontiguousarray(instance_rotation, np.float64)
    rc = None if camera_rotation is None else np.ascontiguousarray(camera_rotation, np.float64)
    r, J = np.zeros(3), np.zeros(18)
    m = f(ORIENTATION_KINDS[kind], _p(t), std, _p(ri), _p(rc), _p(r), _p(J))
    return r[:m].copy(), J[: 6 * m].reshape(m, 6)


RELATIVE_KINDS = {"relative_rotation": 0, "common_position": 1, "linear_motion": 2, "gauge_scale": 3, "heatmap": 4,
                  "relative_motion": 5, "gps_std": 6, "std_deviation": 7, "gps_bias": 8}
REL_PARAMS = 64


def heatmap_residual(grid, width, resolution, x_offset, y_offset, std, instance_pose, rig_camera_pose=None):
    """Heatmap residual and Jacobian [12] (oracle/solver.cpp restatement)."""
    L = lib()
    f = L.oracle_heatmap_residual
    f.argtypes = [D, C.c_int64, C.c_int, C.c_double, D, D, D, D]
    f.restype = C.c_double
    g = np.ascontiguousarray(np.asarray(grid, np.float64).reshape(-1))
    prm = np.array([x_offset, y_offset, std], np.float64)
    pi = np.ascontiguousarray(instance_pose, np.float64)
    pc = None if rig_camera_pose is None else np.ascontiguousarray(rig_camera_pose, np.float64)
    J = np.zeros(12)
    r = f(_p(g), g.size, int(width), float(resolution), _p(prm), _p(pi), _p(pc), _p(J))
    return r, J


def relative_residual(kind: str, instance_poses, params, rig_camera_poses=None, scales=None):
    """Scaled residuals and Jacobian [m][36] of one constraint between shots
    (oracle/solver.cpp restatement); ``scales`` the two reconstruction
    scales of a relative motion (columns 24 and 25), or for "gps_bias" the
    std multiplier (column 24) and the bias rotation, translation and scale
    (columns 12..18)."""
    L = lib()
    f = L.oracle_relative_residual
    f.argtypes = [C.c_int, D, D, D, D, D, D]
    f.restype = C.c_int
    pi = np.ascontiguousarray(instance_poses, np.float64)
    pc = None if rig_camera_poses is None else np.ascontiguousarray(rig_camera_poses, np.float64)
    prm = np.zeros(REL_PARAMS)
    v = np.asarray(params, np.float64).reshape(-1)
    prm[: len(v)] = v
    sc = np.ones(8) if scales is None else np.ascontiguousarray(np.r_[scales, np.ones(8)][:max(8, len(scales))],
                                                                 np.float64)
    r, J = np.zeros(7), np.zeros(7 * 36)
    m = f(RELATIVE_KINDS[kind], _p(pi), _p(pc), _p(prm), _p(sc), _p(r), _p(J))
    return r[:m].copy(), J[: 36 * m].reshape(m, 36)


def depth_residual(instance_pose, point, value, std, radial=True, rig_camera_pose=None):
    """A depth prior's scaled residual and its Jacobian rows (d/d instance
    pose [6], d/d rig camera pose [6], d/d point [3]) (oracle/residuals.h
    restatement of RelativeDepthError).  value and std are used as given."""
    L = lib()
    f = L.oracle_depth_residual
    f.argtypes = [D, D, D, C.c_double, C.c_double, C.c_int, D, D, D]
    f.restype = C.c_double
    pi = np.ascontiguousarray(instance_pose, np.float64)
    pc = None if rig_camera_pose is None else np.ascontiguousarray(rig_camera_pose, np.float64)
    X = np.ascontiguousarray(point, np.float64)
    ji, jr, jp = np.zeros(6), np.zeros(6), np.zeros(3)
    r = f(_p(pi), _p(pc), _p(X), float(value), float(std), 1 if radial else 0, _p(ji), _p(jr), _p(jp))
    return r, ji, jr, jp


def solve(scene, loss=None, irls="mixture", max_iterations=100, gps=True, constant_cameras=False,
          density_ratio=1e-3, skip_initial_reweighting=False, threads=None, orientation=(), relative=(),
          relative_loss=("CauchyLoss", 1.0), gauge=None, heatmap=None, scales=(), fixed_instances=(),
          depth=None, rig_pose=None, bias=None, point_priors=None):
    """Solves the bundle adjustment of a SceneArrays the way
    opensfm_gb300.pybundle.adjuster_from_scene configures the GPU solver.
    ``orientation``: absolute orientation constraints, tuples (kind, shot,
    value, std) with kind one of ORIENTATION_KINDS and value the up vector
    or the angle.  ``relative``: constraints between shots, tuples (kind,
    shots, params) with kind one of RELATIVE_KINDS, shots the 2 (3 for
    linear motion) shot indices and params as gbba_relative_residual takes
    them; ``relative_loss`` the loss of the relative rotations.  ``gauge``:
    (origin shot, scale shot) as set_gauge_fix_shots takes them.
    ``fixed_instances``: rig instances held constant.
    ``heatmap``: (grid, width, resolution), the grid of the ``relative``
    entries of kind "heatmap" (shots (s,), params (x_offset, y_offset,
    std)).  ``scales``: reconstruction scales (value, free) -- the unknowns
    of "relative_motion" entries, whose params are motion[7], the
    observed-scale flag, the 7 x 7 scale matrix, the robust multiplier and
    the two scale indices.  ``depth``: depth priors (observation indices,
    values, stds, radial flags), values and stds rounded to float32 as
    map::Depth stores them.  ``rig_pose``: one fixed rig camera pose
    (angle-axis, centre) composed with every shot (None: the identity, not
    composed).  ``bias``: (rotation, translation, scale, free parameter
    indices) of the one camera's bias, through which every GPS prior is
    taken (kind "gps_bias"; the solved bias is returned as "bias").
    ``point_priors``: (point indices, positions [n][3], stds [n][3]) with
    altitude (GCP3D).  Returns a dict with the final parameters,
    scales, costs and the cost trace."""
    L = lib()
    L.oracle_solve.argtypes = [C.POINTER(_Problem), C.POINTER(_Options), C.POINTER(_Result)]
    L.oracle_solve.restype = C.c_int
    nc = len(scene.camera_projection)
    cam_sigma = np.zeros((nc, 16))
    cam_log = np.zeros((nc, 16), np.uint8)
    for c in range(nc):
        m = int(scene.camera_projection[c])
        s = _SIGMA_ONE[m]
        cam_sigma[c, : len(s)] = s
        cam_log[c, : len(s)] = _LOG[m]
    cam_free = np.zeros((nc, 16), np.uint8)
    for c in range(nc):
        cam_free[c, : num_params(int(scene.camera_projection[c]))] = 0 if constant_cameras else 1
    cam_values = np.ascontiguousarray(scene.camera_values)
    ni = len(scene.rig_instance_poses)
    inst = np.ascontiguousarray(scene.rig_instance_poses)
    inst_free = np.ones((ni, 6), np.uint8)
    for i in fixed_instances:
        inst_free[int(i)] = 0
    has_gps = np.zeros(ni, np.uint8)
    gps_pos = np.zeros((ni, 3))
    gps_std = np.ones((ni, 3))
    bias_terms = []
    if gps and "gps" in scene.extras:
        for s in range(len(scene.shot_camera)):
            i = int(scene.shot_rig_instance[s])
            if bias is not None:
                # the GPS prior through the camera bias: scales 0..6 (after
                # any reconstruction scales) hold the bias
                bias_terms.append(("gps_bias", (s,), np.r_[scene.extras["gps"][s], scene.extras["gps_std"][s], -1.0,
                                                           len(scales) + np.arange(7)]))
                continue
            has_gps[i] = 1
            gps_pos[i] = scene.extras["gps"][s]
            gps_std[i] = scene.extras["gps_std"][s]
    scales = list(scales)
    if bias is not None:
        free = set(int(k) for k in bias[3])
        vals = np.r_[np.asarray(bias[0], np.float64), np.asarray(bias[1], np.float64), float(bias[2])]
        n_before = len(scales)
        scales += [(float(vals[k]), k in free) for k in range(7)]
    rig = np.zeros((1, 6)) if rig_pose is None else np.asarray(rig_pose, np.float64).reshape(1, 6).copy()
    rig_free = np.zeros((1, 6), np.uint8)
    rig_used = np.array([0 if rig_pose is None or not np.any(rig) else 1], np.uint8)
    rig_has_prior = np.ones(1, np.uint8)
    rig_prior = np.zeros((1, 6))
    rig_sigma = np.ones((1, 6))
    ns = len(scene.shot_camera)
    shot_rig = np.zeros(ns, np.int32)
    npt = len(scene.points)
    pts = np.ascontiguousarray(scene.points)
    pfree = np.ones(npt, np.uint8)
    phas = np.zeros(npt, np.uint8)
    pprior = np.zeros((npt, 3))
    psig = np.ones((npt, 3))
    palt = np.ones(npt, np.uint8)
    if point_priors is not None:
        pidx = np.asarray(point_priors[0], np.int64)
        phas[pidx] = 1
        pprior[pidx] = np.asarray(point_priors[1], np.float64)
        psig[pidx] = np.asarray(point_priors[2], np.float64)
    gcp = np.zeros(scene.n_observations, np.uint8)
    no = len(orientation)
    o_kind = np.array([ORIENTATION_KINDS[o[0]] for o in orientation], np.int32).reshape(no)
    o_shot = np.array([int(o[1]) for o in orientation], np.int32).reshape(no)
    o_target = np.zeros((max(no, 1), 3))
    for q, o in enumerate(orientation):
        v = np.atleast_1d(np.asarray(o[2], np.float64))
        o_target[q, : len(v)] = v
    o_std = np.array([float(o[3]) for o in orientation], np.float64).reshape(no)
    relative = list(relative) + bias_terms
    if gauge is not None:
        i0, i1 = (int(scene.shot_rig_instance[int(g)]) for g in gauge)
        inst_free[i0] = 0
        relative.append(("gauge_scale", (int(gauge[0]), int(gauge[1])),
                         [float(np.linalg.norm(inst[i0, 3:] - inst[i1, 3:]))]))
    nr = len(relative)
    r_kind = np.array([RELATIVE_KINDS[c[0]] for c in relative], np.int32).reshape(nr)
    r_shots = np.zeros((max(nr, 1), 3), np.int32)
    r_params = np.zeros((max(nr, 1), REL_PARAMS))
    for q, c in enumerate(relative):
        r_shots[q, : len(c[1])] = c[1]
        v = np.asarray(c[2], np.float64).reshape(-1)
        r_params[q, : len(v)] = v
    keep = [cam_values, cam_sigma, cam_log, cam_free, inst, inst_free, has_gps, gps_pos, gps_std, rig, rig_free,
            rig_used, rig_has_prior, rig_prior, rig_sigma, shot_rig, pts, pfree, phas, pprior, psig, palt, gcp,
            o_kind, o_shot, o_target, o_std, r_kind, r_shots, r_params]
    if heatmap is not None:
        h_grid = np.ascontiguousarray(np.asarray(heatmap[0], np.float64).reshape(-1))
        h_width, h_res = int(heatmap[1]), float(heatmap[2])
    else:
        h_grid, h_width, h_res = np.zeros(1), 1, 1.0
    keep.append(h_grid)
    n_scl = len(scales)
    s_val = np.array([float(v) for v, _ in scales] or [1.0], np.float64)
    s_free = np.array([1 if f else 0 for _, f in scales] or [0], np.uint8)
    keep += [s_val, s_free]
    if depth is not None:
        d_obs = np.ascontiguousarray(depth[0], np.int64)
        d_val = np.asarray(depth[1], np.float32).astype(np.float64)
        d_std = np.asarray(depth[2], np.float32).astype(np.float64)
        d_rad = np.ascontiguousarray(np.broadcast_to(np.asarray(depth[3], np.uint8), d_obs.shape))
    else:
        d_obs, d_val, d_std, d_rad = np.zeros(1, np.int64), np.zeros(1), np.ones(1), np.ones(1, np.uint8)
    n_depth = 0 if depth is None else len(d_obs)
    keep += [d_obs, d_val, d_std, d_rad]
    u8 = lambda a: a.ctypes.data_as(U8)  # noqa: E731
    i32 = lambda a: a.ctypes.data_as(I32)  # noqa: E731
    P = _Problem(nc, i32(scene.camera_projection), _p(cam_values), _p(cam_values.copy() if False else cam_values),
                 _p(cam_sigma), u8(cam_free), u8(cam_log),
                 ni, _p(inst), u8(inst_free), u8(has_gps), _p(gps_pos), _p(gps_std),
                 1, _p(rig), u8(rig_free), u8(rig_used), u8(rig_has_prior), _p(rig_prior), _p(rig_sigma),
                 ns, i32(scene.shot_rig_instance), i32(shot_rig), i32(scene.shot_camera),
                 npt, _p(pts), u8(pfree), u8(phas), _p(pprior), _p(psig), u8(palt),
                 scene.n_observations, i32(scene.obs_shot), i32(scene.obs_point), _p(scene.obs_xy),
                 _p(scene.obs_std), u8(gcp), no, i32(o_kind), i32(o_shot), _p(o_target), _p(o_std),
                 nr, i32(r_kind), i32(r_shots), _p(r_params), LOSSES[relative_loss[0]], float(relative_loss[1]),
                 _p(h_grid), h_grid.size, h_width, h_res, n_scl, _p(s_val), u8(s_free),
                 n_depth, d_obs.ctypes.data_as(C.POINTER(C.c_int64)), _p(d_val), _p(d_std), u8(d_rad))
    loss_kind, loss_a = (0, 1.0) if loss is None else (LOSSES[loss[0]], float(loss[1]))
    O = _Options(max_iterations, loss_kind, loss_a, 1 if irls == "mixture" else 0, density_ratio,
                 int(skip_initial_reweighting), threads or os.cpu_count() or 1)
    out_cam = np.zeros((nc, 16))
    out_inst = np.zeros((ni, 6))
    out_rig = np.zeros((1, 6))
    out_pts = np.zeros((npt, 3))
    out_w = np.zeros(scene.n_observations)
    out_err = np.zeros((scene.n_observations, 3))
    trace = np.zeros(max_iterations + 2)
    out_scl = s_val.copy()
    R = _Result(_p(out_cam), _p(out_inst), _p(out_rig), _p(out_pts), _p(out_scl), _p(out_w), _p(out_err), _p(trace),
                len(trace), 0, 0.0, 0.0, 0, 0, 0)
    if L.oracle_solve(C.byref(P), C.byref(O), C.byref(R)) != 0:
        raise ValueError("oracle_solve: an index array disagrees with the problem's counts")
    del keep
    extra = {} if bias is None else {"bias": out_scl[n_before:n_before + 7].copy()}
    return dict(**extra, cameras=out_cam, instances=out_inst, points=out_pts, scales=out_scl[:n_scl].copy(), weights=out_w,
                errors=out_err,
                trace=trace[: R.trace_n].copy(), initial_cost=R.initial_cost, final_cost=R.final_cost,
                iterations=R.iterations, successful=R.successful, termination=R.termination)


def remove_outliers(errors, weights, obs_point, n_points, filter_type="FIXED", fixed_threshold=0.006,
                    auto_ratio=3.0, weight_threshold=0.5):
    """The observation test of sfm::BAHelpers::RemoveOutliers
    (opensfm/src/lib/sfm/src/ba_helpers.cc:1847-1975) in numpy: the AUTO
    threshold from the componentwise medians (element of rank n/2, as
    std::nth_element at size()/2) and 1.486 x the median deviation norm
    (:1875-1920); outliers by squared error or IRLS weight (:1928-1941);
    points that lose an observation and keep fewer than two (:1958-1967).
    Returns (threshold, outlier flags, removed-point flags)."""
    e = np.asarray(errors, dtype=np.float64)[:, :2]
    w = np.asarray(weights, dtype=np.float64)
    pts = np.asarray(obs_point, dtype=np.int64)
    threshold = 1.0
    if filter_type == "FIXED":
        threshold = float(fixed_threshold)
    elif len(e):
        mid = len(e) // 2
        mx = np.partition(e[:, 0], mid)[mid]
        my = np.partition(e[:, 1], mid)[mid]
        dx = e[:, 0] - mx
        dy = e[:, 1] - my
        dev = np.sqrt(dx * dx + dy * dy)
        robust_std = np.float64(1.486) * np.partition(dev, mid)[mid]
        ax = mx + robust_std
        ay = my + robust_std
        threshold = float(np.float64(auto_ratio) * np.sqrt(ax * ax + ay * ay))
    sq = e[:, 0] * e[:, 0] + e[:, 1] * e[:, 1]
    flags = (sq > np.float64(threshold) * np.float64(threshold)) | (w < weight_threshold)
    counts = np.bincount(pts, minlength=n_points)
    outs = np.bincount(pts[flags], minlength=n_points)
    removed = (outs > 0) & (counts - outs < 2)
    return threshold, flags, removed
