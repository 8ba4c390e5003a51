"""Seeded synthetic bundle-adjustment scenes (numpy, vectorised).

The shapes follow the workloads the bundle adjuster is measured on; the
reference keeps its own seeded generators in opensfm/synthetic_data (circle /
street scenes with pixel noise, GPS noise and perturbed initial poses).

All generators use ``numpy.random.default_rng(seed)`` (PCG64) and return a
:class:`~opensfm_gb300.scene.SceneArrays` whose ``extras`` hold the ground
truth and the generation parameters.  Observations are normalized image
coordinates (pixel offset from the image centre divided by max(width,
height), geometry/camera.h:90-96) and carry ``obs_std`` in the same units.
"""
from __future__ import annotations

import numpy as np

from .scene import (BROWN, DUAL, FISHEYE, FISHEYE62, FISHEYE624, FISHEYE_OPENCV, PERSPECTIVE,
                    RADIAL, SIMPLE_RADIAL, SPHERICAL, SceneArrays)

# ---------------------------------------------------------------------------
# rotations


def rotation_matrix(aa: np.ndarray) -> np.ndarray:
    """Rodrigues rotation matrices [..., 3, 3] of angle-axis vectors [..., 3]."""
    aa = np.asarray(aa, np.float64)
    th = np.linalg.norm(aa, axis=-1, keepdims=True)
    k = np.where(th > 0, aa / np.where(th > 0, th, 1.0), 0.0)
    K = np.zeros(aa.shape[:-1] + (3, 3))
    K[..., 0, 1], K[..., 0, 2] = -k[..., 2], k[..., 1]
    K[..., 1, 0], K[..., 1, 2] = k[..., 2], -k[..., 0]
    K[..., 2, 0], K[..., 2, 1] = -k[..., 1], k[..., 0]
    s = np.sin(th)[..., None]
    c = np.cos(th)[..., None]
    eye = np.broadcast_to(np.eye(3), K.shape)
    return eye + s * K + (1 - c) * (K @ K)


def rotation_vector(Rm: np.ndarray) -> np.ndarray:
    """Angle-axis vectors of rotation matrices [..., 3, 3].

    Goes through a unit quaternion built with Shepperd's method (the largest
    of w, x, y, z is computed from the diagonal), which stays accurate for
    angles near pi."""
    Rm = np.asarray(Rm, np.float64)
    shape = Rm.shape[:-2]
    M = Rm.reshape(-1, 3, 3)
    tr = M[:, 0, 0] + M[:, 1, 1] + M[:, 2, 2]
    cand = np.stack([tr, M[:, 0, 0], M[:, 1, 1], M[:, 2, 2]], axis=-1)
    k = np.argmax(cand, axis=-1)
    q = np.zeros((len(M), 4))
    for case in range(4):
        m = k == case
        if not np.any(m):
            continue
        A = M[m]
        if case == 0:
            s = np.sqrt(1.0 + tr[m]) * 2
            q[m] = np.stack([0.25 * s, (A[:, 2, 1] - A[:, 1, 2]) / s, (A[:, 0, 2] - A[:, 2, 0]) / s,
                             (A[:, 1, 0] - A[:, 0, 1]) / s], -1)
        elif case == 1:
            s = np.sqrt(1.0 + A[:, 0, 0] - A[:, 1, 1] - A[:, 2, 2]) * 2
            q[m] = np.stack([(A[:, 2, 1] - A[:, 1, 2]) / s, 0.25 * s, (A[:, 0, 1] + A[:, 1, 0]) / s,
                             (A[:, 0, 2] + A[:, 2, 0]) / s], -1)
        elif case == 2:
            s = np.sqrt(1.0 + A[:, 1, 1] - A[:, 0, 0] - A[:, 2, 2]) * 2
            q[m] = np.stack([(A[:, 0, 2] - A[:, 2, 0]) / s, (A[:, 0, 1] + A[:, 1, 0]) / s, 0.25 * s,
                             (A[:, 1, 2] + A[:, 2, 1]) / s], -1)
        else:
            s = np.sqrt(1.0 + A[:, 2, 2] - A[:, 0, 0] - A[:, 1, 1]) * 2
            q[m] = np.stack([(A[:, 1, 0] - A[:, 0, 1]) / s, (A[:, 0, 2] + A[:, 2, 0]) / s,
                             (A[:, 1, 2] + A[:, 2, 1]) / s, 0.25 * s], -1)
    q *= np.where(q[:, :1] < 0, -1.0, 1.0)
    v = q[:, 1:]
    n = np.linalg.norm(v, axis=-1)
    ang = 2 * np.arctan2(n, q[:, 0])
    f = np.where(n > 1e-15, ang / np.where(n > 1e-15, n, 1.0), 2.0)
    return (v * f[:, None]).reshape(shape + (3,))


def look_at(centres: np.ndarray, targets: np.ndarray, up=(0.0, 0.0, 1.0)) -> np.ndarray:
    """World-to-camera rotations of cameras at centres looking at targets
    (camera z forward, x right, y down)."""
    z = targets - centres
    z /= np.linalg.norm(z, axis=-1, keepdims=True)
    up = np.broadcast_to(np.asarray(up, np.float64), z.shape)
    x = np.cross(z, up)
    bad = np.linalg.norm(x, axis=-1) < 1e-9
    if np.any(bad):
        x[bad] = np.cross(z[bad], np.array([0.0, 1.0, 0.0]))
    x /= np.linalg.norm(x, axis=-1, keepdims=True)
    y = np.cross(z, x)
    return np.stack([x, y, z], axis=-2)


def pose_from_rotation(R_wc: np.ndarray, centres: np.ndarray) -> np.ndarray:
    """bundle::Pose data [rx, ry, rz, tx, ty, tz] (camera-to-world angle-axis,
    camera centre) of world-to-camera rotations and centres."""
    r = rotation_vector(np.swapaxes(R_wc, -1, -2))
    return np.concatenate([r, centres], axis=-1)


def world_to_camera(poses: np.ndarray, X: np.ndarray) -> np.ndarray:
    """x_cam = R(-r) (X - c) for pose rows matched with point rows."""
    Rwc = np.swapaxes(rotation_matrix(poses[..., :3]), -1, -2)
    return np.einsum("...ij,...j->...i", Rwc, X - poses[..., 3:6])


# ---------------------------------------------------------------------------
# camera models (forward maps only; used to synthesise observations)


def _distort(model: int, q: np.ndarray, k: np.ndarray) -> np.ndarray:
    x, y = q[..., 0], q[..., 1]
    r2 = x * x + y * y
    if model in (PERSPECTIVE, FISHEYE, DUAL, RADIAL):
        rad = 1 + r2 * (k[..., 0] + k[..., 1] * r2)
        return q * rad[..., None]
    if model == SIMPLE_RADIAL:
        return q * (1 + r2 * k[..., 0])[..., None]
    if model == FISHEYE_OPENCV:
        rad = 1 + r2 * (k[..., 0] + r2 * (k[..., 1] + r2 * (k[..., 2] + r2 * k[..., 3])))
        return q * rad[..., None]
    if model == BROWN:
        rad = 1 + r2 * (k[..., 0] + r2 * (k[..., 1] + r2 * k[..., 2]))
        p1, p2 = k[..., 3], k[..., 4]
    else:  # FISHEYE62 / FISHEYE624
        rad = 1 + r2 * (k[..., 0] + r2 * (k[..., 1] + r2 * (k[..., 2] + r2 * (
            k[..., 3] + r2 * (k[..., 4] + r2 * k[..., 5])))))
        p1, p2 = k[..., 6], k[..., 7]
    tx = 2 * p1 * x * y + p2 * (r2 + 2 * x * x)
    ty = 2 * p2 * x * y + p1 * (r2 + 2 * y * y)
    if model == FISHEYE624:
        tx = tx + k[..., 8] * r2 + k[..., 9] * r2 * r2
        ty = ty + k[..., 10] * r2 + k[..., 11] * r2 * r2
    return np.stack([x * rad + tx, y * rad + ty], axis=-1)


def project(model: int, params: np.ndarray, p: np.ndarray) -> np.ndarray:
    """Projects camera-frame points p [..., 3] with one camera model."""
    x, y, z = p[..., 0], p[..., 1], p[..., 2]
    if model == SPHERICAL:
        lon = np.arctan2(x, z)
        lat = np.arctan2(-y, np.sqrt(x * x + z * z))
        return np.stack([lon, -lat], axis=-1) / (2 * np.pi)
    if model in (FISHEYE, FISHEYE_OPENCV, FISHEYE62, FISHEYE624, DUAL):
        r = np.sqrt(x * x + y * y)
        th = np.arctan2(r, z)
        f = np.where(r > 0, th / np.where(r > 0, r, 1.0), 1.0)
        a = np.stack([f * x, f * y], axis=-1)
        if model == DUAL:
            t = params[..., 0]
            pp = np.stack([x / z, y / z], axis=-1)
            a = t[..., None] * pp + (1 - t[..., None]) * a
    else:
        a = np.stack([x / z, y / z], axis=-1)
    n_proj = 1 if model == DUAL else 0
    nd = {PERSPECTIVE: 2, BROWN: 5, FISHEYE: 2, FISHEYE_OPENCV: 4, FISHEYE62: 8, FISHEYE624: 12,
          DUAL: 2, RADIAL: 2, SIMPLE_RADIAL: 1}[model]
    b = _distort(model, a, params[..., n_proj:n_proj + nd])
    af = params[..., n_proj + nd:]
    if model in (PERSPECTIVE, FISHEYE, DUAL):
        return b * af[..., 0:1]
    return np.stack([af[..., 0] * b[..., 0] + af[..., 2], af[..., 0] * af[..., 1] * b[..., 1] + af[..., 3]],
                    axis=-1)


def project_scene(scene: SceneArrays, poses: np.ndarray, points: np.ndarray) -> np.ndarray:
    """Projections of every observation of scene with given poses and points."""
    sh = scene.obs_shot
    Rwc = np.swapaxes(rotation_matrix(poses[:, :3]), -1, -2)  # per instance
    inst = scene.shot_rig_instance[sh]
    pc = np.einsum("nij,nj->ni", Rwc[inst], points[scene.obs_point] - poses[inst, 3:6])
    cams = scene.shot_camera[sh]
    out = np.zeros((len(sh), 2))
    for c in np.unique(cams):
        m = cams == c
        model = int(scene.camera_projection[c])
        out[m] = project(model, np.broadcast_to(scene.camera_values[c], (int(m.sum()), 16)), pc[m])
    return out


def _perturb_poses(rng, poses, rot_sigma, trans_sigma):
    out = poses.copy()
    if rot_sigma > 0:
        dR = rotation_matrix(rng.normal(0, rot_sigma, (len(poses), 3)))
        out[:, :3] = rotation_vector(dR @ rotation_matrix(poses[:, :3]))
    out[:, 3:] += rng.normal(0, trans_sigma, (len(poses), 3))
    return out


# ---------------------------------------------------------------------------
# scenes


def ring_scene(seed: int = 42, n_shots: int = 20, n_points: int = 2000, obs_per_point: int = 6,
               radius: float = 10.0, cube: float = 4.0, model: int = PERSPECTIVE,
               params=(-0.1, 0.01, 0.85), width: int = 1000, height: int = 750,
               pixel_noise: float = 1.0, rot_sigma: float = 0.01, trans_sigma: float = 0.1,
               point_sigma: float = 0.05, outlier_ratio: float = 0.0) -> SceneArrays:
    """Cameras on a horizontal ring looking inward at points in a cube.

    Default: 20 perspective cameras (focal 0.85, k1 -0.1, k2 0.01) on a 10 m
    ring, 2,000 points uniform in a 4 m cube, each seen by 6 cameras
    (12k observations), 1 px Gaussian noise at 1000x750, initial poses
    perturbed by 0.01 rad / 0.1 m and points by 0.05 m."""
    rng = np.random.default_rng(seed)
    ang = np.linspace(0, 2 * np.pi, n_shots, endpoint=False)
    centres = np.stack([radius * np.cos(ang), radius * np.sin(ang), 0.3 * np.sin(3 * ang)], axis=-1)
    R_wc = look_at(centres, np.zeros_like(centres))
    poses = pose_from_rotation(R_wc, centres)
    pts = rng.uniform(-cube / 2, cube / 2, (n_points, 3))
    k = min(obs_per_point, n_shots)
    shots = np.argsort(rng.random((n_points, n_shots)), axis=1)[:, :k]
    obs_point = np.repeat(np.arange(n_points, dtype=np.int32), k)
    obs_shot = shots.reshape(-1).astype(np.int32)
    scale = 1.0 / max(width, height)
    scene = SceneArrays(
        camera_projection=[model], camera_values=np.asarray([params], np.float64),
        rig_instance_poses=poses, shot_rig_instance=np.arange(n_shots), shot_camera=np.zeros(n_shots),
        points=pts, obs_shot=obs_shot, obs_point=obs_point,
        obs_xy=np.zeros((len(obs_shot), 2)), obs_std=np.full(len(obs_shot), pixel_noise * scale))
    xy = project_scene(scene, poses, pts)
    xy += rng.normal(0, pixel_noise * scale, xy.shape)
    if outlier_ratio > 0:
        bad = rng.random(len(xy)) < outlier_ratio
        xy[bad, 0] = rng.uniform(-0.5 * width * scale, 0.5 * width * scale, bad.sum())
        xy[bad, 1] = rng.uniform(-0.5 * height * scale, 0.5 * height * scale, bad.sum())
    scene.obs_xy = np.ascontiguousarray(xy)
    scene.extras = dict(true_poses=poses, true_points=pts, seed=seed, width=width, height=height)
    scene.rig_instance_poses = _perturb_poses(rng, poses, rot_sigma, trans_sigma)
    scene.points = pts + rng.normal(0, point_sigma, pts.shape)
    return scene


def depth_priors(scene: SceneArrays, fraction: float = 0.3, std: float = 0.05, radial: bool = True,
                 noise: float = 0.02, seed: int = 0):
    """Depth priors (map::Depth) on a seeded share of a scene's
    observations: the true depth of the observed point in the camera (its
    camera-frame z, or its distance when radial) plus Gaussian noise.
    Returns (observation indices, values, stds, radial flags) as
    BundleAdjuster.set_depth_priors takes them."""
    rng = np.random.default_rng(seed)
    idx = np.nonzero(rng.random(scene.n_observations) < fraction)[0].astype(np.int64)
    poses = scene.extras["true_poses"][scene.shot_rig_instance[scene.obs_shot[idx]]]
    pc = world_to_camera(poses, scene.extras["true_points"][scene.obs_point[idx]])
    d = np.linalg.norm(pc, axis=-1) if radial else pc[:, 2]
    value = d + rng.normal(0.0, noise, len(idx))
    return idx, value, np.full(len(idx), std), np.full(len(idx), radial, np.uint8)


def _geometric_lengths(rng, n, mean, lo, hi):
    # track lengths >= lo with geometric tail of the given mean
    p = 1.0 / max(mean - lo + 1, 1.0)
    return np.clip(lo - 1 + rng.geometric(p, n), lo, hi)


def street_scene(seed: int = 7, n_shots: int = 500, n_points: int = 200_000, mean_track: float = 7.0,
                 n_cameras: int = 4, outlier_ratio: float = 0.02, width: int = 1000, height: int = 750,
                 pixel_noise: float = 1.0, rot_sigma: float = 0.002, trans_sigma: float = 0.05,
                 point_sigma: float = 0.05) -> SceneArrays:
    """Brown cameras along a random-walk street trajectory.

    Default: 500 shots (1 m steps, smooth heading changes) sharing 4 Brown
    camera models, 200k points on the street facades and ground, geometric
    track lengths of mean 7 (~1.4M observations), 2% outliers uniform over
    the image."""
    rng = np.random.default_rng(seed)
    heading = np.cumsum(rng.normal(0, 0.03, n_shots))
    step = np.stack([np.cos(heading), np.sin(heading)], axis=-1)
    xy = np.cumsum(step, axis=0)
    centres = np.concatenate([xy, np.full((n_shots, 1), 2.0)], axis=-1)
    # cameras alternate between forward and slightly side-looking
    yaw = heading + rng.choice([-0.35, -0.12, 0.12, 0.35], n_shots)
    fwd = np.stack([np.cos(yaw), np.sin(yaw), np.full(n_shots, -0.05)], axis=-1)
    R_wc = look_at(centres, centres + fwd)
    poses = pose_from_rotation(R_wc, centres)
    cams = np.zeros((n_cameras, 9))
    for c in range(n_cameras):
        cams[c] = [-0.08 + 0.02 * c, 0.01, -0.001, 0.0005 * (c - 1.5), -0.0004, 0.8 + 0.03 * c,
                   1.0 + 0.002 * c, 0.002 * (c - 1.5), -0.003]
    shot_cam = np.arange(n_shots) % n_cameras
    # points: anchored at a random shot, placed in its view
    anchor = rng.integers(0, n_shots, n_points)
    u = rng.uniform(-0.45, 0.45, n_points)
    v = rng.uniform(-0.3, 0.3, n_points)
    depth = rng.uniform(6.0, 30.0, n_points)
    ray = np.stack([u / 0.85, v / 0.85, np.ones(n_points)], axis=-1) * depth[:, None]
    pts = centres[anchor] + np.einsum("nji,nj->ni", R_wc[anchor], ray)
    L = _geometric_lengths(rng, n_points, mean_track, 2, 40)
    scale = 1.0 / max(width, height)
    obs_s, obs_p = [], []
    count = np.zeros(n_points, np.int64)
    alive = np.ones(n_points, bool)
    for off in [0] + [s * o for o in range(1, 60) for s in (1, -1)]:
        sh = anchor + off
        ok = alive & (sh >= 0) & (sh < n_shots) & (count < L)
        if not np.any(ok):
            continue
        idx = np.nonzero(ok)[0]
        s_idx = sh[idx]
        pc = world_to_camera(poses[s_idx], pts[idx])
        front = pc[:, 2] > 1.0
        proj = pc[:, :2] / np.where(front, pc[:, 2], 1.0)[:, None]
        vis = front & (np.abs(proj[:, 0]) < 0.48) & (np.abs(proj[:, 1]) < 0.36)
        idx, s_idx = idx[vis], s_idx[vis]
        obs_s.append(s_idx)
        obs_p.append(idx)
        count[idx] += 1
    obs_shot = np.concatenate(obs_s).astype(np.int32)
    obs_point = np.concatenate(obs_p).astype(np.int32)
    keep_pt = count >= 2
    remap = np.full(n_points, -1, np.int64)
    remap[keep_pt] = np.arange(keep_pt.sum())
    m = keep_pt[obs_point]
    obs_shot, obs_point = obs_shot[m], remap[obs_point[m]].astype(np.int32)
    pts = pts[keep_pt]
    order = np.lexsort((obs_shot, obs_point))
    obs_shot, obs_point = obs_shot[order], obs_point[order]
    scene = SceneArrays(
        camera_projection=[BROWN] * n_cameras, camera_values=cams, rig_instance_poses=poses,
        shot_rig_instance=np.arange(n_shots), shot_camera=shot_cam, points=pts, obs_shot=obs_shot,
        obs_point=obs_point, obs_xy=np.zeros((len(obs_shot), 2)),
        obs_std=np.full(len(obs_shot), pixel_noise * scale))
    xy_obs = project_scene(scene, poses, pts) + rng.normal(0, pixel_noise * scale, (len(obs_shot), 2))
    bad = rng.random(len(xy_obs)) < outlier_ratio
    xy_obs[bad, 0] = rng.uniform(-0.5, 0.5, bad.sum())
    xy_obs[bad, 1] = rng.uniform(-0.375, 0.375, bad.sum())
    scene.obs_xy = np.ascontiguousarray(xy_obs)
    scene.extras = dict(true_poses=poses, true_points=pts, true_cameras=cams.copy(), outliers=bad,
                        seed=seed)
    scene.rig_instance_poses = _perturb_poses(rng, poses, rot_sigma, trans_sigma)
    scene.points = pts + rng.normal(0, point_sigma, pts.shape)
    return scene


def aerial_scene(seed: int = 3, nx: int = 70, ny: int = 72, n_points: int = 2_000_000,
                 mean_track: float = 8.6, altitude: float = 120.0, forward_overlap: float = 0.8,
                 side_overlap: float = 0.7, focal: float = 0.85, width: int = 1000, height: int = 750,
                 offset=(5.0e5, 4.0e6, 0.0), gps_sigma=(2.0, 2.0, 4.0), pixel_noise: float = 1.0,
                 rot_sigma: float = 0.002, trans_sigma: float = 0.5, point_sigma: float = 0.3) -> SceneArrays:
    """Nadir perspective cameras on a grid over sinusoidal terrain.

    Default: 70 x 72 = 5,040 cameras at 120 m with 80% forward / 70% side
    overlap, 2M ground points, per-point track lengths geometric with mean
    8.6 (before the visibility cut) among the cameras that see the point (~15M observations), and per-shot
    GPS priors with sigma (2, 2, 4) m, all in UTM-scale coordinates
    (x ~ 5e5, y ~ 4e6)."""
    rng = np.random.default_rng(seed)
    half_w = 0.5 * altitude / focal                       # ground half-width (x)
    half_h = half_w * height / width                      # ground half-height (y)
    dx = 2 * half_w * (1 - side_overlap)
    dy = 2 * half_h * (1 - forward_overlap)
    gx, gy = np.meshgrid(np.arange(nx) * dx, np.arange(ny) * dy, indexing="ij")
    n_shots = nx * ny
    off = np.asarray(offset, np.float64)

    def terrain(x, y):
        return 8.0 * np.sin(x / 150.0) * np.cos(y / 110.0) + 3.0 * np.sin(x / 37.0 + y / 53.0)

    cx, cy = gx.reshape(-1), gy.reshape(-1)
    centres = np.stack([cx, cy, np.full(n_shots, altitude)], axis=-1)
    # nadir: camera z points down; x along +x world; small per-shot jitter
    base = np.array([[1.0, 0.0, 0.0], [0.0, -1.0, 0.0], [0.0, 0.0, -1.0]])
    jitter = rotation_matrix(rng.normal(0, 0.02, (n_shots, 3)))
    R_wc = jitter @ base
    centres_w = centres + off
    poses = pose_from_rotation(R_wc, centres_w)
    # points on the terrain over the covered area
    px = rng.uniform(-half_w * 0.8, (nx - 1) * dx + half_w * 0.8, n_points)
    py = rng.uniform(-half_h * 0.8, (ny - 1) * dy + half_h * 0.8, n_points)
    pts_local = np.stack([px, py, terrain(px, py)], axis=-1)
    # candidate cameras: grid cells around the point
    ix = np.rint(px / dx).astype(np.int64)
    iy = np.rint(py / dy).astype(np.int64)
    reach_x = int(np.ceil(half_w / dx)) + 1
    reach_y = int(np.ceil(half_h / dy)) + 1
    L = _geometric_lengths(rng, n_points, mean_track, 2, 30)
    cand_s, cand_p, cand_key = [], [], []
    scale = 1.0 / max(width, height)
    for ox in range(-reach_x, reach_x + 1):
        for oy in range(-reach_y, reach_y + 1):
            sx, sy = ix + ox, iy + oy
            ok = (sx >= 0) & (sx < nx) & (sy >= 0) & (sy < ny)
            idx = np.nonzero(ok)[0]
            s = (sx[idx] * ny + sy[idx]).astype(np.int64)
            pc = np.einsum("nij,nj->ni", R_wc[s], pts_local[idx] - centres[s])
            proj = pc[:, :2] / pc[:, 2:3]
            # focal-scaled bound: |f * proj| < 0.49 (normalized image half-size)
            vis = (pc[:, 2] > 1.0) & (np.abs(focal * proj[:, 0]) < 0.49) & \
                  (np.abs(focal * proj[:, 1]) < 0.49 * height / width)
            cand_s.append(s[vis])
            cand_p.append(idx[vis])
            cand_key.append(rng.random(int(vis.sum())))
    cs = np.concatenate(cand_s)
    cp = np.concatenate(cand_p)
    ck = np.concatenate(cand_key)
    order = np.lexsort((ck, cp))
    cs, cp = cs[order], cp[order]
    first = np.searchsorted(cp, np.arange(n_points))
    rank = np.arange(len(cp)) - first[cp]
    keep = rank < L[cp]
    cs, cp = cs[keep], cp[keep]
    cnt = np.bincount(cp, minlength=n_points)
    keep_pt = cnt >= 2
    remap = np.full(n_points, -1, np.int64)
    remap[keep_pt] = np.arange(keep_pt.sum())
    m = keep_pt[cp]
    obs_shot = cs[m].astype(np.int32)
    obs_point = remap[cp[m]].astype(np.int32)
    pts_w = pts_local[keep_pt] + off
    cams = np.array([[-0.05, 0.005, focal]])
    scene = SceneArrays(
        camera_projection=[PERSPECTIVE], camera_values=cams, rig_instance_poses=poses,
        shot_rig_instance=np.arange(n_shots), shot_camera=np.zeros(n_shots), points=pts_w,
        obs_shot=obs_shot, obs_point=obs_point, obs_xy=np.zeros((len(obs_shot), 2)),
        obs_std=np.full(len(obs_shot), pixel_noise * scale))
    xy_obs = project_scene(scene, poses, pts_w) + rng.normal(0, pixel_noise * scale, (len(obs_shot), 2))
    scene.obs_xy = np.ascontiguousarray(xy_obs)
    gs = np.asarray(gps_sigma, np.float64)
    gps = centres_w + rng.normal(0, 1, (n_shots, 3)) * gs
    scene.extras = dict(true_poses=poses, true_points=pts_w, gps=gps, gps_std=np.tile(gs, (n_shots, 1)),
                        seed=seed, offset=off)
    scene.rig_instance_poses = _perturb_poses(rng, poses, rot_sigma, trans_sigma)
    scene.points = pts_w + rng.normal(0, point_sigma, pts_w.shape)
    return scene


def random_model_params(model: int, rng=None) -> np.ndarray:
    """Plausible camera parameters of a model (geometry::Camera order)."""
    rng = rng or np.random.default_rng(0)
    f = 0.5 + 0.3 * rng.random()
    if model == PERSPECTIVE or model == FISHEYE:
        return np.array([-0.05, 0.01, f])
    if model == BROWN:
        return np.array([-0.1, 0.03, 0.001, 0.001, 0.002, f, 1.01, 0.01, -0.02])
    if model == FISHEYE_OPENCV:
        return np.array([-0.1, 0.03, 0.001, 0.005, f, 1.0, 0.01, -0.02])
    if model == FISHEYE62:
        return np.array([-0.1, 0.03, 0.001, 0.005, 0.02, 0.001, 0.0007, -0.01, f, 1.0, 0.01, -0.02])
    if model == FISHEYE624:
        return np.array([-0.1, 0.03, 0.001, 0.005, 0.02, 0.001, 0.0007, -0.01, 0.01, -0.007, -0.03,
                         0.0053, f, 1.0, 0.01, -0.02])
    if model == SPHERICAL:
        return np.array([0.0])
    if model == DUAL:
        return np.array([0.5, -0.05, 0.01, f])
    if model == RADIAL:
        return np.array([0.1, 0.03, f, 1.0, 0.01, -0.02])
    if model == SIMPLE_RADIAL:
        return np.array([0.1, f, 1.0, 0.01, -0.02])
    raise ValueError(model)


def random_scene(seed: int, models, n_shots: int = 12, n_points: int = 300, obs_per_point: int = 4,
                 rig: bool = False) -> SceneArrays:
    """Small random scene mixing camera models (and optionally rig cameras):
    parity-test material, not a benchmark workload."""
    rng = np.random.default_rng(seed)
    models = list(models)
    cams = np.zeros((len(models), 16))
    for i, m in enumerate(models):
        v = random_model_params(m, rng)
        cams[i, : len(v)] = v
    ang = np.linspace(0, 2 * np.pi, n_shots, endpoint=False) + rng.normal(0, 0.05, n_shots)
    centres = np.stack([6 * np.cos(ang), 6 * np.sin(ang), rng.normal(0, 0.3, n_shots)], axis=-1)
    R_wc = look_at(centres, rng.normal(0, 0.3, (n_shots, 3)))
    poses = pose_from_rotation(R_wc, centres)
    pts = rng.uniform(-1.5, 1.5, (n_points, 3))
    k = min(obs_per_point, n_shots)
    shots = np.argsort(rng.random((n_points, n_shots)), axis=1)[:, :k]
    obs_point = np.repeat(np.arange(n_points), k).astype(np.int32)
    obs_shot = shots.reshape(-1).astype(np.int32)
    kw = {}
    if rig:
        n_rc = 2
        rc = np.zeros((n_rc, 6))
        rc[1] = [0.02, -0.03, 0.01, 0.1, 0.0, 0.05]
        rc[0] = [0.0, 0.0, 0.0, 0.0, 0.0, 0.0]
        kw = dict(rig_camera_poses=rc, rig_camera_used=np.array([1, 1], np.uint8),
                  shot_rig_camera=(np.arange(n_shots) % n_rc).astype(np.int32))
    scene = SceneArrays(camera_projection=models, camera_values=cams, rig_instance_poses=poses,
                        shot_rig_instance=np.arange(n_shots), shot_camera=np.arange(n_shots) % len(models),
                        points=pts, obs_shot=obs_shot, obs_point=obs_point,
                        obs_xy=rng.uniform(-0.3, 0.3, (len(obs_shot), 2)),
                        obs_std=rng.uniform(0.5e-3, 2e-3, len(obs_shot)), **kw)
    return scene


def local_ba_problems(n_problems: int = 256, seed: int = 23, shots=(5, 60), points=(500, 20_000),
                      observations=(3_000, 150_000), models=(BROWN, FISHEYE, SPHERICAL)) -> list:
    """Uneven local bundle adjustments: per problem, shots, points and
    observations drawn log-uniformly from the given ranges and one camera
    model from `models`; ring geometry (ring_scene) with 1 px noise and
    perturbed initial poses and points."""
    rng = np.random.default_rng(seed)

    def lu(lo, hi):
        return float(np.exp(rng.uniform(np.log(lo), np.log(hi))))

    out = []
    for q in range(n_problems):
        n_shots = int(round(lu(*shots)))
        n_points = int(round(lu(*points)))
        n_obs = lu(*observations)
        k = int(np.clip(round(n_obs / n_points), 2, n_shots))
        model = int(models[rng.integers(len(models))])
        params = tuple(random_model_params(model, rng))
        out.append(ring_scene(seed=int(rng.integers(1 << 30)), n_shots=n_shots, n_points=n_points,
                              obs_per_point=k, model=model, params=params))
    return out


def projection_scene(n_obs: int, model: int, seed: int = 17, n_shots: int = 64, obs_per_point: int = 4,
                     n_cameras: int = 4) -> SceneArrays:
    """Large scene for the differentiable projection operator: n_shots
    cameras of one model (n_cameras intrinsics sets) on a ring looking at a
    cube of points, each point seen by obs_per_point random shots;
    observations are the exact projections plus 1 px noise."""
    rng = np.random.default_rng(seed)
    n_points = max(1, n_obs // obs_per_point)
    cams = np.zeros((n_cameras, 16))
    for i in range(n_cameras):
        v = random_model_params(model, rng)
        cams[i, : len(v)] = v
    ang = np.linspace(0, 2 * np.pi, n_shots, endpoint=False) + rng.normal(0, 0.05, n_shots)
    centres = np.stack([6 * np.cos(ang), 6 * np.sin(ang), rng.normal(0, 0.3, n_shots)], axis=-1)
    poses = pose_from_rotation(look_at(centres, rng.normal(0, 0.3, (n_shots, 3))), centres)
    pts = rng.uniform(-1.5, 1.5, (n_points, 3))
    obs_point = np.repeat(np.arange(n_points), obs_per_point).astype(np.int32)[:n_obs]
    obs_shot = rng.integers(0, n_shots, len(obs_point)).astype(np.int32)
    shot_camera = (np.arange(n_shots) % n_cameras).astype(np.int32)
    scene = SceneArrays(camera_projection=np.full(n_cameras, model), camera_values=cams, rig_instance_poses=poses,
                        shot_rig_instance=np.arange(n_shots), shot_camera=shot_camera, points=pts,
                        obs_shot=obs_shot, obs_point=obs_point, obs_xy=np.zeros((len(obs_shot), 2)),
                        obs_std=np.full(len(obs_shot), 1e-3))
    from .scene import evaluate_projections
    from . import _lib as lib
    # exact projections (residuals at zero observations, scaled by std),
    # then noise
    r = evaluate_projections(scene, lib.PRECISION_FP64).residuals
    scene.obs_xy = np.ascontiguousarray(r[:, :2] * 1e-3 + rng.normal(0, 1e-3, (len(obs_shot), 2)))
    return scene
