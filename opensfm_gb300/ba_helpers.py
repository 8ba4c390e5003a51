"""Local bundle adjustment around shots: the neighbourhood selection and
the problem set-up of ``sfm::BAHelpers::BundleLocal``
(opensfm/src/lib/sfm/src/ba_helpers.cc:64-440), on the flat scene arrays
of :mod:`opensfm_gb300.scene`, driving the GPU adjuster.

* :func:`shot_neighborhood` -- ``ShotNeighborhood`` / ``DirectShotNeighbors``
  (ba_helpers.cc:64-136): the interior grows from the central shots (and
  their rig-instance siblings) by ``radius - 1`` hops over shots sharing at
  least ``min_common_points`` points, most shared points first, up to
  ``max_interior_size`` shots; the boundary is every other shot that sees a
  point of the interior.  Ties in the shared-point count are broken by shot
  index (the reference's ``std::sort`` leaves their order unspecified).
* :func:`select_tracks_grid` -- ``SelectTracksGrid`` (ba_helpers.cc:
  938-1004): in every interior shot's image, a grid_size x grid_size grid
  keeps the longest track (most observations) per cell that no earlier shot
  selected; the other tracks seen from the interior are returned for
  retriangulation.  Shots are visited in index order and observations in
  scene order (the reference iterates a hash set).
* :func:`local_problem` -- the set-up of ``BundleLocal`` (ba_helpers.cc:
  176-330): cameras and rig cameras fixed; the rig instances of interior and
  boundary shots, fixed when one of their shots is on the boundary; the
  averaged GPS of an instance's interior shots as its position prior; the
  grid-selected tracks (``local_bundle_grid``, default 12) with all their
  observations.  Without image sizes, or with grid_size <= 1, every track
  seen from the interior is taken (the reference would take none).
* :func:`bundle_local` -- one local bundle solved and written back.
* :func:`bundle_local_batch` -- many local bundles at once: the problems
  the batched solver takes (no position priors) go through one
  :class:`~opensfm_gb300.pybundle.BundleBatch` solve (one captured LM
  iteration for all of them), the others run one at a time.  Results are
  written back in the order of ``central_shots`` (a shot in several
  interiors keeps the last one's pose).

* :func:`shot_poses_problem` / :func:`bundle_shot_poses` --
  ``BundleShotPoses`` (ba_helpers.cc): the poses of the given shots alone --
  cameras, rig cameras and every point they see held constant, an instance
  fixed when one of its shots is not among them, averaged GPS on the free
  instances, the given shots' observations, 10 iterations with exact
  (``DENSE_QR``) steps.
* :func:`bundle_stochastic` -- ``BundleStochastic`` (ba_helpers.cc:
  1231-1370): K = min(ceil(3 S / N), max_rounds) rounds, each a local
  bundle around ``random_shots`` seeds drawn by a partial Fisher-Yates
  shuffle of the shots, with the stochastic radius and an interior budget
  of N shots; every round starts from the previous round's result.  The
  seeds come from numpy's generator (the reference's ``std::mt19937(42)``
  draws differ); GCP-anchored seeds and the GPS-bias compensation of
  ``BundleLocalStochastic`` are not applied.
* :func:`bundle_full` -- ``BundleFull`` (ba_helpers.cc:1372-1671): the
  whole scene with grid-selected tracks, optimised cameras, averaged GPS,
  up-vector priors when the alignment is an orientation prior, ground
  control points and the GPS-bias compensation, written back by
  :func:`bundle_to_map` (``BundleToMap``, :1673-1736: NaN / Inf refused).
* :func:`bundle_local_stochastic` -- ``BundleLocalStochastic``
  (ba_helpers.cc:442-804): a local bundle with fixed cameras, the
  GPS-bias compensation (every GPS-bearing instance as a fixed anchor) and
  ground control points.
* Ground control points: :class:`GroundControlPoint`,
  :func:`triangulate_gcp` (``TriangulateGCP``), :func:`add_gcp_to_bundle`
  (``AddGCPToBundle``), :func:`determine_gcp_bias_parameters`,
  :func:`detect_alignment_constraints`.  Positions are in the scene's
  (topocentric) frame; the reference converts latitude, longitude and
  altitude first.  Retriangulation of the unselected tracks stays with the
  caller (it is sfm::retriangulation, outside the adjuster).

Defaults are the reference's configuration values (opensfm/config.py:
``local_bundle_radius`` 3, ``local_bundle_min_common_points`` 20,
``local_bundle_max_shots`` 30, ``stochastic_bundle_max_shots`` 500,
``stochastic_bundle_random_shots`` 20, ``stochastic_bundle_radius`` 100,
``stochastic_bundle_max_rounds`` 100).
"""
from __future__ import annotations

import copy
import math
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Sequence, Set, Tuple

import numpy as np

from . import pybundle
from .pygeometry import Camera, Pose, Similarity
from .scene import NUM_PARAMS, SceneArrays


@dataclass
class Covisibility:
    """Shot <-> point incidence of a scene (each pair once)."""
    shot_points: List[np.ndarray]
    point_shots: List[np.ndarray]
    instance_shots: Dict[int, List[int]]
    shot_instance: np.ndarray

    @classmethod
    def of(cls, scene: SceneArrays) -> "Covisibility":
        n_shots = len(scene.shot_camera)
        n_points = len(scene.points)
        pairs = np.unique(np.stack([np.asarray(scene.obs_shot, np.int64), np.asarray(scene.obs_point, np.int64)], 1),
                          axis=0)
        by_shot = np.argsort(pairs[:, 0], kind="stable")
        sp = np.split(pairs[by_shot, 1], np.searchsorted(pairs[by_shot, 0], np.arange(1, n_shots)))
        by_point = np.lexsort((pairs[:, 0], pairs[:, 1]))
        ps = np.split(pairs[by_point, 0], np.searchsorted(pairs[by_point, 1], np.arange(1, n_points)))
        inst = np.asarray(scene.shot_rig_instance, np.int64)
        instance_shots: Dict[int, List[int]] = {}
        for s in range(n_shots):
            instance_shots.setdefault(int(inst[s]), []).append(s)
        return cls(sp, ps, instance_shots, inst)


def direct_shot_neighbors(cov: Covisibility, shots: Set[int], min_common_points: int,
                          max_neighbors: int) -> Set[int]:
    """DirectShotNeighbors (ba_helpers.cc:95-136): shots outside ``shots``
    that see at least ``min_common_points`` of their points, most first, at
    most ``max_neighbors`` of them, each with its rig-instance siblings."""
    points = set()
    for s in shots:
        points.update(cov.shot_points[s].tolist())
    common: Dict[int, int] = {}
    for p in points:
        for s in cov.point_shots[p].tolist():
            if s not in shots:
                common[s] = common.get(s, 0) + 1
    pairs = sorted(common.items(), key=lambda kv: (-kv[1], kv[0]))
    max_n = min(max_neighbors, len(pairs))
    neighbors: Set[int] = set()
    for idx, (s, n) in enumerate(pairs):
        if n >= min_common_points and idx < max_n:
            neighbors.update(cov.instance_shots[int(cov.shot_instance[s])])
        else:
            break
    return neighbors


def shot_neighborhood(cov: Covisibility, central_shots: Sequence[int], radius: int = 3,
                      min_common_points: int = 20, max_interior_size: int = 30) -> Tuple[Set[int], Set[int]]:
    """ShotNeighborhood (ba_helpers.cc:64-93): (interior, boundary)."""
    interior: Set[int] = set()
    for c in central_shots:
        interior.update(cov.instance_shots[int(cov.shot_instance[c])])
        interior.add(int(c))
    distance = 1
    while distance < radius and len(interior) < max_interior_size:
        interior |= direct_shot_neighbors(cov, interior, min_common_points, max_interior_size - len(interior))
        distance += 1
    boundary = direct_shot_neighbors(cov, interior, 1, 1_000_000)
    return interior, boundary


def select_tracks_grid(scene: SceneArrays, cov: Covisibility, shots: Set[int], grid_size: int, width: int,
                       height: int) -> Tuple[np.ndarray, np.ndarray]:
    """SelectTracksGrid (ba_helpers.cc:938-1004): (selected tracks, other
    tracks seen from ``shots``), as sorted point indices."""
    if not shots or grid_size <= 1 or width <= 0 or height <= 0:
        return np.zeros(0, np.int64), np.zeros(0, np.int64)
    obs_shot = np.asarray(scene.obs_shot)
    obs_point = np.asarray(scene.obs_point)
    xy = np.asarray(scene.obs_xy)
    track_len = np.array([len(ps) for ps in cov.point_shots], np.int64)
    normalize = max(width, height)
    order = np.argsort(obs_shot, kind="stable")
    starts = np.searchsorted(obs_shot[order], np.arange(len(scene.shot_camera) + 1))
    selected: Set[int] = set()
    seen: Set[int] = set()
    for s in sorted(shots):
        cells: Dict[int, Tuple[int, int]] = {}
        for o in order[starts[s]:starts[s + 1]]:
            p = int(obs_point[o])
            seen.add(p)
            x = min(1.0, max(0.0, (xy[o, 0] * normalize + width * 0.5) / width))
            y = min(1.0, max(0.0, (xy[o, 1] * normalize + height * 0.5) / height))
            gx = min(int(x * grid_size), grid_size - 1)
            gy = min(int(y * grid_size), grid_size - 1)
            cell = gx + gy * grid_size
            best = cells.get(cell, (-1, 0))
            if track_len[p] > best[1] and p not in selected:
                cells[cell] = (p, int(track_len[p]))
        selected.update(p for p, _ in cells.values())
    return (np.array(sorted(selected), np.int64), np.array(sorted(seen - selected), np.int64))


@dataclass
class LocalProblem:
    """A local bundle set up on a scene."""
    adjuster: pybundle.BundleAdjuster
    interior: Set[int]
    boundary: Set[int]
    point_ids: np.ndarray                  # scene point indices in the problem
    free_instances: List[int] = field(default_factory=list)
    has_position_priors: bool = False
    other_tracks: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int64))  # to retriangulate


def local_problem(scene: SceneArrays, central_shots: Sequence[int], cov: Optional[Covisibility] = None,
                  radius: int = 3, min_common_points: int = 20, max_shots: int = 30, use_gps: bool = True,
                  precision: str = "mixed", loss: Optional[tuple] = None, max_iterations: int = 10,
                  linear_solver: Optional[str] = None, grid_size: int = 12, image_size: Optional[Tuple[int, int]] = None
                  ) -> LocalProblem:
    """The local bundle of ``BundleLocal`` around ``central_shots``.
    ``image_size`` (width, height) for the track grid; by default the
    scene's ``extras`` width and height when present."""
    cov = cov or Covisibility.of(scene)
    interior, boundary = shot_neighborhood(cov, central_shots, radius, min_common_points, max_shots)
    shots = sorted(interior | boundary)
    ba = pybundle.BundleAdjuster()
    ba.set_precision(precision)
    ba.set_max_num_iterations(max_iterations)
    if linear_solver is not None:
        ba.set_linear_solver_type(linear_solver)
    if loss is not None:
        ba.set_point_projection_loss_function(*loss)
    used_cameras = sorted({int(scene.shot_camera[s]) for s in shots})
    for c in used_cameras:
        m = int(scene.camera_projection[c])
        cam = Camera(m, scene.camera_values[c, : NUM_PARAMS[m]])
        ba.add_camera(str(c), cam, cam, True)
    ba.add_rig_camera("rig", Pose(), Pose(), True)
    gps = scene.extras.get("gps") if use_gps else None
    gps_std = scene.extras.get("gps_std") if use_gps else None
    free_instances, has_priors = [], False
    for inst in sorted({int(cov.shot_instance[s]) for s in shots}):
        members = cov.instance_shots[inst]
        fixed = any(s in boundary for s in members)
        pose = Pose.from_ba_data(scene.rig_instance_poses[inst])
        ba.add_rig_instance(str(inst), pose, {str(s): str(int(scene.shot_camera[s])) for s in members},
                            {str(s): "rig" for s in members}, fixed)
        if not fixed:
            free_instances.append(inst)
            if gps is not None:
                inner = [s for s in members if s in interior]
                if inner:
                    ba.add_rig_instance_position_prior(str(inst), np.mean([gps[s] for s in inner], axis=0),
                                                       np.mean([gps_std[s] for s in inner], axis=0), "")
                    has_priors = True
    if image_size is None and "width" in scene.extras and "height" in scene.extras:
        image_size = (int(scene.extras["width"]), int(scene.extras["height"]))
    other_tracks = np.zeros(0, np.int64)
    if image_size is not None and grid_size > 1:
        point_ids, other_tracks = select_tracks_grid(scene, cov, interior, grid_size, *image_size)
    else:
        point_ids = np.unique(np.concatenate([cov.shot_points[s] for s in sorted(interior)]) if interior
                              else np.zeros(0, np.int64))
    # every observation of these points (their shots are all in interior or boundary)
    keep = np.isin(np.asarray(scene.obs_point), point_ids)
    local_index = -np.ones(len(scene.points), np.int64)
    local_index[point_ids] = np.arange(len(point_ids))
    ba.add_points(scene.points[point_ids])
    shot_index = {s: ba.shot_index(str(s)) for s in shots}
    obs_shot = np.array([shot_index[int(s)] for s in np.asarray(scene.obs_shot)[keep]], np.int32)
    ba.add_point_projection_observations(obs_shot, local_index[np.asarray(scene.obs_point)[keep]].astype(np.int32),
                                         np.asarray(scene.obs_xy)[keep], np.asarray(scene.obs_std)[keep])
    return LocalProblem(ba, interior, boundary, point_ids, free_instances, has_priors, other_tracks)


def _write_back(scene: SceneArrays, lp: LocalProblem, poses: np.ndarray, points: np.ndarray) -> None:
    for inst in lp.free_instances:
        poses[inst] = lp.adjuster.get_rig_instance_pose(str(inst)).ba_data()
    points[lp.point_ids] = lp.adjuster.get_points()


def bundle_local(scene: SceneArrays, central_shot: int, **kw) -> Tuple[np.ndarray, np.ndarray, LocalProblem]:
    """One local bundle around ``central_shot`` on the GPU; returns the
    scene's rig-instance poses and points with the local solution written
    in, and the problem (its adjuster holds the summary)."""
    lp = local_problem(scene, [central_shot], **kw)
    lp.adjuster.run()
    poses, points = np.array(scene.rig_instance_poses, copy=True), np.array(scene.points, copy=True)
    _write_back(scene, lp, poses, points)
    return poses, points, lp


def bundle_local_batch(scene: SceneArrays, central_shots: Sequence[int], batch_precision: str = "mixed",
                       batch_pcg_iterations: int = 50, batch_pcg_tolerance: float = 1e-3,
                       **kw) -> Tuple[np.ndarray, np.ndarray, List[LocalProblem]]:
    """Local bundles around each of ``central_shots``: those without
    position priors solved together as one batched GPU solve, the rest one
    at a time.  Returns the updated poses and points and the problems."""
    cov = Covisibility.of(scene)
    problems = [local_problem(scene, [c], cov=cov, **kw) for c in central_shots]
    batched = [lp for lp in problems if not lp.has_position_priors]
    if batched:
        batch = pybundle.BundleBatch()
        batch.set_options(precision=batch_precision, max_iterations=kw.get("max_iterations", 10),
                          pcg_iterations=batch_pcg_iterations, pcg_tolerance=batch_pcg_tolerance)
        for lp in batched:
            batch.add(lp.adjuster)
        batch.run()
    for lp in problems:
        if lp.has_position_priors:
            lp.adjuster.run()
    poses, points = np.array(scene.rig_instance_poses, copy=True), np.array(scene.points, copy=True)
    for lp in problems:
        _write_back(scene, lp, poses, points)
    return poses, points, problems


def shot_poses_problem(scene: SceneArrays, shot_ids: Sequence[int], cov: Optional[Covisibility] = None,
                       use_gps: bool = True, precision: str = "mixed", loss: Optional[tuple] = None,
                       max_iterations: int = 10) -> LocalProblem:
    """The problem of BundleShotPoses for ``shot_ids`` (its ``interior``;
    the boundary is empty: every point is held)."""
    cov = cov or Covisibility.of(scene)
    chosen = {int(s) for s in shot_ids}
    instances = sorted({int(cov.shot_instance[s]) for s in chosen})
    ba = pybundle.BundleAdjuster()
    ba.set_precision(precision)
    ba.set_max_num_iterations(max_iterations)
    ba.set_linear_solver_type("DENSE_QR")
    if loss is not None:
        ba.set_point_projection_loss_function(*loss)
    members_of = {i: cov.instance_shots[i] for i in instances}
    shots = sorted({s for i in instances for s in members_of[i]})
    for c in sorted({int(scene.shot_camera[s]) for s in shots}):
        m = int(scene.camera_projection[c])
        cam = Camera(m, scene.camera_values[c, : NUM_PARAMS[m]])
        ba.add_camera(str(c), cam, cam, True)
    ba.add_rig_camera("rig", Pose(), Pose(), True)
    gps = scene.extras.get("gps") if use_gps else None
    gps_std = scene.extras.get("gps_std") if use_gps else None
    free_instances, has_priors = [], False
    for inst in instances:
        members = members_of[inst]
        fixed = any(s not in chosen for s in members)
        ba.add_rig_instance(str(inst), Pose.from_ba_data(scene.rig_instance_poses[inst]),
                            {str(s): str(int(scene.shot_camera[s])) for s in members},
                            {str(s): "rig" for s in members}, fixed)
        if not fixed:
            free_instances.append(inst)
            if gps is not None:
                ba.add_rig_instance_position_prior(str(inst), np.mean([gps[s] for s in members], axis=0),
                                                   np.mean([gps_std[s] for s in members], axis=0), "")
                has_priors = True
    point_ids = np.unique(np.concatenate([cov.shot_points[s] for s in sorted(chosen)]) if chosen
                          else np.zeros(0, np.int64))
    local_index = -np.ones(len(scene.points), np.int64)
    local_index[point_ids] = np.arange(len(point_ids))
    ba.add_points(scene.points[point_ids], np.ones(len(point_ids), np.uint8))
    keep = np.isin(np.asarray(scene.obs_shot), sorted(chosen))
    shot_index = {s: ba.shot_index(str(s)) for s in shots}
    obs_shot = np.array([shot_index[int(s)] for s in np.asarray(scene.obs_shot)[keep]], np.int32)
    ba.add_point_projection_observations(obs_shot, local_index[np.asarray(scene.obs_point)[keep]].astype(np.int32),
                                         np.asarray(scene.obs_xy)[keep], np.asarray(scene.obs_std)[keep])
    return LocalProblem(ba, chosen, set(), point_ids, free_instances, has_priors)


def bundle_shot_poses(scene: SceneArrays, shot_ids: Sequence[int], **kw) -> Tuple[np.ndarray, LocalProblem]:
    """BundleShotPoses on the GPU: the given shots' rig-instance poses
    refined against constant points; returns the scene's poses with them
    written in, and the problem."""
    lp = shot_poses_problem(scene, shot_ids, **kw)
    lp.adjuster.run()
    poses = np.array(scene.rig_instance_poses, copy=True)
    for inst in lp.free_instances:
        poses[inst] = lp.adjuster.get_rig_instance_pose(str(inst)).ba_data()
    return poses, lp


def stochastic_rounds(num_shots: int, max_shots: int = 500, max_rounds: int = 100) -> Tuple[int, int]:
    """(rounds, interior budget) of BundleStochastic (ba_helpers.cc:
    1246-1266): P(a shot is adjusted at least once) ~ 1 - exp(-K N / S),
    K = ceil(3 S / N) for about 95% coverage, capped at ``max_rounds``."""
    n = max(1, min(max_shots, num_shots))
    k = int(math.ceil(3.0 * num_shots / n))
    return max(1, min(k, max_rounds)), n


def stochastic_seeds(rng: np.random.Generator, shot_ids: List[int], random_shots: int) -> List[int]:
    """The round's seeds: a partial Fisher-Yates shuffle of ``shot_ids``
    (in place, carried over rounds), its first ``random_shots`` entries."""
    k = max(1, min(random_shots, len(shot_ids)))
    seeds = []
    for i in range(k):
        j = int(rng.integers(i, len(shot_ids)))
        shot_ids[i], shot_ids[j] = shot_ids[j], shot_ids[i]
        seeds.append(shot_ids[i])
    return seeds


def bundle_stochastic(scene: SceneArrays, max_shots: int = 500, random_shots: int = 20, radius: int = 100,
                      max_rounds: int = 100, seed: int = 42, **kw) -> Tuple[np.ndarray, np.ndarray, dict]:
    """BundleStochastic: rounds of local bundles around random seeds, each
    starting from the previous round's poses and points.  Returns the final
    poses and points and a report (rounds, seeds and summaries)."""
    n_shots = len(scene.shot_camera)
    rounds, budget = stochastic_rounds(n_shots, max_shots, max_rounds)
    rng = np.random.default_rng(seed)
    ids = list(range(n_shots))
    work = copy.copy(scene)
    work.rig_instance_poses = np.array(scene.rig_instance_poses, copy=True)
    work.points = np.array(scene.points, copy=True)
    cov = Covisibility.of(scene)
    report = {"num_rounds": rounds, "interior_budget": budget, "rounds": []}
    for _ in range(rounds):
        seeds = stochastic_seeds(rng, ids, random_shots)
        lp = local_problem(work, seeds, cov=cov, radius=radius, max_shots=budget, **kw)
        lp.adjuster.run()
        _write_back(work, lp, work.rig_instance_poses, work.points)
        report["rounds"].append({"seeds": seeds, "interior": len(lp.interior), "points": int(len(lp.point_ids)),
                                 "summary": lp.adjuster.summary()})
    return work.rig_instance_poses, work.points, report


# ---------------------------------------------------------------------------
# Full bundle, stochastic local bundles, ground control points, write-back
# (BundleFull ba_helpers.cc:1372-1671, BundleLocalStochastic :442-804,
# TriangulateGCP / AddGCPToBundle :822-936, AlignmentConstraints /
# DetectAlignmentConstraints :1738-1802, DetermineGCPBiasParameters
# :1804-1845, BundleToMap :1673-1736).

# The configuration values the helpers read, with the reference's defaults
# (opensfm/config.py).
DEFAULT_CONFIG = {
    "optimize_camera_parameters": True, "optimize_rig_parameters": False, "bundle_use_gps": True,
    "bundle_use_gcp": True, "bundle_compensate_gps_bias": False, "gcp_reprojection_error_threshold": 0.05,
    "gcp_global_weight": 0.04, "gcp_observation_sd": 0.001, "gcp_horizontal_sd": 0.01, "gcp_vertical_sd": 0.1,
    "align_method": "auto", "align_orientation_prior": "horizontal", "exif_focal_sd": 0.01,
    "aspect_ratio_sd": 0.01, "principal_point_sd": 0.01, "radial_distortion_k1_sd": 0.01,
    "radial_distortion_k2_sd": 0.01, "tangential_distortion_p1_sd": 0.01, "tangential_distortion_p2_sd": 0.01,
    "radial_distortion_k3_sd": 0.01, "radial_distortion_k4_sd": 0.01, "rig_translation_sd": 0.1,
    "rig_rotation_sd": 0.1, "bundle_irls_density_ratio": 0.001, "bundle_irls_gcp_density_ratio": 0.00001,
    "bundle_irls_gps_density_ratio": 0.00001, "bundle_max_iterations": 100, "local_bundle_radius": 3,
    "local_bundle_min_common_points": 20, "local_bundle_max_shots": 30, "local_bundle_grid": 12,
    "final_bundle_grid": 32,
    # not a reference key: the two-level PCG preconditioner's cluster size
    # for bundles solved by PCG (0: block-Jacobi only, as Ceres'
    # SCHUR_JACOBI); it acts only once a linear solve needs many iterations
    "bundle_coarse_leaf": 32,
}


def _config(config: Optional[dict]) -> dict:
    c = dict(DEFAULT_CONFIG)
    c.update(config or {})
    return c


@dataclass
class GroundControlPoint:
    """map::GroundControlPoint: observations (shot index, normalized image
    point) and, unless only observed, the measured position in the scene's
    (topocentric) frame -- the reference converts its latitude, longitude
    and altitude with the map's topocentric converter first -- with an
    optional standard deviation.  Check points take no part in the
    adjustment."""
    id: str
    observations: List[Tuple[int, np.ndarray]]
    position: Optional[np.ndarray] = None
    std_dev: Optional[np.ndarray] = None
    has_altitude: bool = True
    role: str = "control"


def determine_linear_solver(num_cameras: int) -> str:
    """DetermineLinearSolver (ba_helpers.cc:42-49)."""
    return "DENSE_SCHUR" if num_cameras <= 200 else "SPARSE_SCHUR"


def are_points_collinear(X: np.ndarray) -> bool:
    """ArePointsCollinear (ba_helpers.cc:26-40): two eigenvalues of the
    scatter below 1e-10, or the largest over the middle above 5e3."""
    X = np.asarray(X, float)
    Z = X - X.mean(axis=0)
    ev = np.linalg.eigvalsh(Z.T @ Z)
    return int(np.sum(ev < 1e-10)) > 1 or abs(ev[2] / ev[1]) > 5e3


def _shot_frame(scene: SceneArrays, shot: int) -> Tuple[np.ndarray, np.ndarray]:
    """(camera-to-world rotation, camera centre) of a shot."""
    pose = Pose.from_ba_data(scene.rig_instance_poses[int(scene.shot_rig_instance[shot])])
    return pose.get_R_cam_to_world(), pose.get_origin()


def _angle(a: np.ndarray, b: np.ndarray) -> float:
    c = np.dot(a, b) / (np.linalg.norm(a) * np.linalg.norm(b))
    return float(np.arccos(np.clip(c, -1.0, 1.0)))


def triangulate_gcp(gcp: GroundControlPoint, scene: SceneArrays, threshold: float, min_ray_angle: float = 0.1 * math.pi / 180,
                    min_depth: float = 1e-3, iterations: int = 10) -> Tuple[bool, np.ndarray, np.ndarray]:
    """TriangulateGCP (ba_helpers.cc:822-857) with the steps of
    TriangulateBearingsRobust (geometry/src/triangulation.cc:239-302): world
    bearings of the observations from existing shots; some pair of rays
    between min_ray_angle and pi - min_ray_angle; the midpoint solution
    (least squares over the rays); inliers within `threshold` radians of
    their ray, at least two; refinement of the bearing errors over the
    inliers (Gauss-Newton, `iterations` steps); every inlier at least
    min_depth in front.  The reference samples ray pairs by RANSAC; here
    the inliers come from the all-ray solution, re-solved on them once, a
    deterministic choice that agrees on outlier-free control points.
    Returns (success, position, inlier flags)."""
    n_shots = len(scene.shot_camera)
    cams = [Camera(int(scene.camera_projection[c]), scene.camera_values[c, : NUM_PARAMS[int(scene.camera_projection[c])]])
            for c in range(len(scene.camera_projection))]
    centres, bearings = [], []
    for shot, xy in gcp.observations:
        if not 0 <= int(shot) < n_shots:
            continue
        R, c = _shot_frame(scene, int(shot))
        centres.append(c)
        bearings.append(R @ cams[int(scene.shot_camera[int(shot)])].bearing(xy))
    n = len(centres)
    if n < 2:
        return False, np.zeros(3), np.zeros(n, bool)
    C_, B_ = np.array(centres), np.array(bearings)
    B_ = B_ / np.linalg.norm(B_, axis=1, keepdims=True)
    if not any(min_ray_angle <= _angle(B_[i], B_[j]) <= math.pi - min_ray_angle
               for i in range(n) for j in range(i)):
        return False, np.zeros(3), np.zeros(n, bool)

    def midpoint(idx):
        A, b = np.zeros((3, 3)), np.zeros(3)
        for i in idx:
            P = np.eye(3) - np.outer(B_[i], B_[i])
            A += P
            b += P @ C_[i]
        return np.linalg.lstsq(A, b, rcond=None)[0]

    X = midpoint(range(n))
    inl = np.array([_angle(X - C_[i], B_[i]) <= threshold for i in range(n)])
    if inl.sum() < 2:
        return False, np.zeros(3), inl
    X = midpoint(np.nonzero(inl)[0])
    idx = np.nonzero(inl)[0]
    for _ in range(iterations):
        # residual: the component of the normalized ray to X orthogonal to the bearing
        J, r = [], []
        for i in idx:
            d = X - C_[i]
            nd = np.linalg.norm(d)
            u = d / nd
            P = np.eye(3) - np.outer(B_[i], B_[i])
            r.append(P @ u)
            J.append(P @ (np.eye(3) - np.outer(u, u)) / nd)
        J, r = np.concatenate(J), np.concatenate(r)
        step = np.linalg.lstsq(J, -r, rcond=None)[0]
        X = X + step
        if np.linalg.norm(step) < 1e-12 * (1.0 + np.linalg.norm(X)):
            break
    for i in idx:
        if np.dot(X - C_[i], B_[i]) < min_depth:
            return False, np.zeros(3), inl
    return True, X, inl


def add_gcp_to_bundle(ba: pybundle.BundleAdjuster, scene: SceneArrays, gcps: Sequence[GroundControlPoint],
                      config: dict, num_ba_points: int, num_ba_shots: int, ba_shots: Set[int]) -> int:
    """AddGCPToBundle (ba_helpers.cc:860-936): each triangulated control
    point seen from a shot of the problem becomes a point "gcp-<id>" with a
    prior at its measured position (std / (gcp_global_weight * w)) and its
    observations as GCP projections (std gcp_observation_sd / (weight *
    w)), w = sqrt(max(1, points per shot)).  Returns the observations
    added."""
    c = _config(config)
    weight = c["gcp_global_weight"] * math.sqrt(max(1.0, num_ba_points / max(1, num_ba_shots)))
    added = 0
    for g in gcps:
        if g.role == "checkpoint":
            continue
        ok, X, _ = triangulate_gcp(g, scene, c["gcp_reprojection_error_threshold"])
        if not ok or not any(int(s) in ba_shots for s, _ in g.observations):
            continue
        pid = "gcp-" + g.id
        ba.add_point(pid, X, False)
        if g.position is not None:
            sd = (np.asarray(g.std_dev, float) if g.std_dev is not None else
                  np.array([c["gcp_horizontal_sd"], c["gcp_horizontal_sd"], c["gcp_vertical_sd"]]))
            ba.add_point_prior(pid, np.asarray(g.position, float), sd / weight, g.has_altitude)
        for s, xy in g.observations:
            if int(s) in ba_shots:
                ba.add_point_projection_observation(str(int(s)), pid, np.asarray(xy, float),
                                                    c["gcp_observation_sd"] / weight, True)
                added += 1
    return added


def alignment_constraints(scene: SceneArrays, gcps: Sequence[GroundControlPoint], config: dict
                          ) -> Tuple[np.ndarray, np.ndarray]:
    """AlignmentConstraints (ba_helpers.cc:1738-1787): measured (Xp) and
    reconstructed (X) positions of the triangulated control points and of
    the shots with GPS."""
    c = _config(config)
    Xp, X = [], []
    if c["bundle_use_gcp"]:
        for g in gcps:
            if g.position is None:
                continue
            ok, pos, _ = triangulate_gcp(g, scene, c["gcp_reprojection_error_threshold"])
            if ok:
                Xp.append(np.asarray(g.position, float))
                X.append(pos)
    if c["bundle_use_gps"] and "gps" in scene.extras:
        for s in range(len(scene.shot_camera)):
            Xp.append(np.asarray(scene.extras["gps"][s], float))
            X.append(_shot_frame(scene, s)[1])
    return np.array(Xp).reshape(-1, 3), np.array(X).reshape(-1, 3)


def detect_alignment_constraints(scene: SceneArrays, gcps: Sequence[GroundControlPoint], config: dict) -> str:
    """DetectAlignmentConstraints (ba_helpers.cc:1789-1802)."""
    _, X = alignment_constraints(scene, gcps, config)
    if len(X) < 3 or are_points_collinear(X):
        return "orientation_prior"
    return "naive"


def determine_gcp_bias_parameters(scene: SceneArrays, gcps: Sequence[GroundControlPoint], config: dict) -> List[int]:
    """DetermineGCPBiasParameters (ba_helpers.cc:1804-1845) as
    SimilarityMaskToIndices gives it (bundle/data/parameter_mask.h:42-62):
    every parameter without triangulated control points or with three or
    more not collinear; the translation for one; translation and scale for
    two or collinear ones."""
    c = _config(config)
    pts = []
    for g in gcps:
        ok, X, _ = triangulate_gcp(g, scene, c["gcp_reprojection_error_threshold"])
        if ok:
            pts.append(X)
    if not pts:
        return list(range(7))
    if len(pts) == 1:
        return [3, 4, 5]
    if len(pts) == 2 or are_points_collinear(np.array(pts)):
        return [3, 4, 5, 6]
    return list(range(7))


def _configure(ba: pybundle.BundleAdjuster, c: dict, n_shots: int) -> None:
    ba.set_internal_parameters_prior_sd(c["exif_focal_sd"], c["aspect_ratio_sd"], c["principal_point_sd"],
                                        c["radial_distortion_k1_sd"], c["radial_distortion_k2_sd"],
                                        c["tangential_distortion_p1_sd"], c["tangential_distortion_p2_sd"],
                                        c["radial_distortion_k3_sd"], c["radial_distortion_k4_sd"])
    ba.set_rig_parameters_prior_sd(c["rig_translation_sd"], c["rig_rotation_sd"])
    ba.set_default_density_ratio(c["bundle_irls_density_ratio"])
    ba.set_group_density_ratio("GCP2D", c["bundle_irls_gcp_density_ratio"])
    ba.set_group_density_ratio("GPS", c["bundle_irls_gps_density_ratio"])
    ba.set_max_num_iterations(int(c["bundle_max_iterations"]))
    if int(c.get("bundle_coarse_leaf", 0)) > 0:
        ba.set_coarse_preconditioner(int(c["bundle_coarse_leaf"]))


def _up_vector(scene: SceneArrays, gcps, c: dict) -> Optional[np.ndarray]:
    method = c["align_method"]
    if method == "auto":
        method = detect_alignment_constraints(scene, gcps, c)
    if method == "orientation_prior":
        if c["align_orientation_prior"] == "vertical":
            return np.array([0.0, 0.0, -1.0])
        if c["align_orientation_prior"] == "horizontal":
            return np.array([0.0, -1.0, 0.0])
    return None


def _instance_gps(scene: SceneArrays, members: Sequence[int]) -> Optional[Tuple[np.ndarray, np.ndarray]]:
    """The averaged GPS position and accuracy of an instance's shots; an
    accuracy component <= 0 is an error (ba_helpers.cc:1500-1510)."""
    if "gps" not in scene.extras:
        return None
    pos, acc = [], []
    for s in members:
        a = np.asarray(scene.extras["gps_std"][s], float)
        if np.any(a <= 0):
            raise RuntimeError(f"Shot {s} has an accuracy component <= 0. Try modifying your input parser to "
                               "filter such values.")
        pos.append(np.asarray(scene.extras["gps"][s], float))
        acc.append(a)
    return np.mean(pos, axis=0), np.mean(acc, axis=0)


def bundle_to_map(ba: pybundle.BundleAdjuster, scene: SceneArrays, update_cameras: bool,
                  instances: Optional[Sequence[int]] = None, point_ids: Optional[np.ndarray] = None,
                  biases: bool = True) -> Dict[str, np.ndarray]:
    """BundleToMap (ba_helpers.cc:1673-1736) on the scene arrays: cameras
    (when updated), biases and rig-instance poses, each refused with a
    RuntimeError when it holds NaN or Inf; points written back, and a point
    with a non-finite position gets unit reprojection errors and zero
    weights.  Returns the reprojection errors and weights of the written
    points' observations ("errors", "weights", per scene observation; NaN
    where not written)."""
    if update_cameras:
        for c in range(len(scene.camera_projection)):
            cam = ba.get_camera(str(c))
            scene.camera_values[c, : len(cam.get_parameters_values())] = cam.get_parameters_values()
    if biases:
        out = scene.extras.setdefault("biases", {})
        for c in range(len(scene.camera_projection)):
            b = ba.get_bias(str(c))
            if not b.is_valid():
                raise RuntimeError(f"Bias {c} has either NaN or INF values.")
            out[str(c)] = b
    inst = range(len(scene.rig_instance_poses)) if instances is None else instances
    for i in inst:
        d = ba.get_rig_instance_pose(str(i)).ba_data()
        if not np.all(np.isfinite(d)):
            raise RuntimeError(f"Rig Instance {i} has either NaN or INF values.")
        scene.rig_instance_poses[i] = d
    ids = np.arange(len(scene.points)) if point_ids is None else np.asarray(point_ids)
    pts = ba.get_points()[: len(ids)]
    errors = np.full((scene.n_observations, 3), np.nan)
    weights = np.full(scene.n_observations, np.nan)
    try:
        e, w, _ = ba.projection_results()
    except Exception:  # reprojection errors not computed
        e, w = None, None
    if e is not None and len(e) >= 1:
        # the adjuster's observations are the scene observations of these
        # points, in scene order (the helpers add them so)
        keep = np.nonzero(np.isin(np.asarray(scene.obs_point), ids))[0]
        m = min(len(keep), len(e))
        errors[keep[:m]] = e[:m]
        weights[keep[:m]] = w[:m]
    bad = ~np.all(np.isfinite(pts), axis=1)
    if bad.any():
        obs_bad = np.isin(np.asarray(scene.obs_point), ids[bad])
        errors[obs_bad] = 1.0
        weights[obs_bad] = 0.0
    scene.points[ids] = pts
    return {"errors": errors, "weights": weights}


def _add_scene_shots(ba: pybundle.BundleAdjuster, scene: SceneArrays, cov: Covisibility, instances: Sequence[int],
                     fixed: Set[int], use_gps: bool, gps_on_fixed: bool) -> List[int]:
    moving = []
    for inst in instances:
        members = cov.instance_shots[inst]
        f = inst in fixed
        ba.add_rig_instance(str(inst), Pose.from_ba_data(scene.rig_instance_poses[inst]),
                            {str(s): str(int(scene.shot_camera[s])) for s in members},
                            {str(s): "rig" for s in members}, f)
        if not f:
            moving.append(inst)
        if use_gps and (not f or gps_on_fixed):
            g = _instance_gps(scene, members)
            if g is not None:
                ba.add_rig_instance_position_prior(str(inst), g[0], g[1], "dummy")
    return moving


def bundle_full(scene: SceneArrays, config: Optional[dict] = None, gcps: Sequence[GroundControlPoint] = (),
                grid_size: Optional[int] = None, camera_priors: Optional[Sequence[Camera]] = None,
                precision: str = "mixed") -> dict:
    """BundleFull (ba_helpers.cc:1372-1671) on the GPU adjuster: the tracks
    of SelectTracksGrid over every shot (grid_size <= 1 or no image size:
    every point), cameras optimised unless optimize_camera_parameters is
    off, rig instances with their averaged GPS, an up-vector prior per shot
    when the alignment is an orientation prior, ground control points, the
    GPS-bias compensation (every camera's bias with
    determine_gcp_bias_parameters' parameters) when asked and control
    points exist, the configuration's priors and IRLS density ratios, the
    linear solver of determine_linear_solver; then the solution written
    back (bundle_to_map).  Retriangulation of the other tracks is the
    caller's.  Returns the report (brief, full and IRLS reports, wall
    times, counts, the other tracks)."""
    import time
    c = _config(config)
    t0 = time.perf_counter()
    cov = Covisibility.of(scene)
    n_shots = len(scene.shot_camera)
    grid = c["final_bundle_grid"] if grid_size is None else grid_size
    width, height = scene.extras.get("width"), scene.extras.get("height")
    if width and height and grid > 1:
        subset, other = select_tracks_grid(scene, cov, set(range(n_shots)), grid, int(width), int(height))
    else:
        subset, other = np.arange(len(scene.points)), np.zeros(0, np.int64)
    t_grid = time.perf_counter()
    ba = pybundle.BundleAdjuster()
    ba.set_precision(precision)
    fix_cameras = not c["optimize_camera_parameters"]
    for k in range(len(scene.camera_projection)):
        m = int(scene.camera_projection[k])
        cam = Camera(m, scene.camera_values[k, : NUM_PARAMS[m]])
        prior = camera_priors[k] if camera_priors is not None else cam
        ba.add_camera(str(k), cam, prior, fix_cameras)
    ba.add_points(scene.points[subset])
    up = _up_vector(scene, gcps, c)
    ba.add_rig_camera("rig", Pose(), Pose(), True)
    _add_scene_shots(ba, scene, cov, sorted(cov.instance_shots), set(), bool(c["bundle_use_gps"]), False)
    if up is not None:
        for s in range(n_shots):
            ba.add_absolute_up_vector(str(s), up, 1e-3)
    keep = np.nonzero(np.isin(np.asarray(scene.obs_point), subset))[0]
    local = -np.ones(len(scene.points), np.int64)
    local[subset] = np.arange(len(subset))
    shot_index = np.array([ba.shot_index(str(s)) for s in range(n_shots)], np.int32)
    ba.add_point_projection_observations(shot_index[np.asarray(scene.obs_shot)[keep]],
                                         local[np.asarray(scene.obs_point)[keep]].astype(np.int32),
                                         np.asarray(scene.obs_xy)[keep], np.asarray(scene.obs_std)[keep])
    if c["bundle_use_gcp"] and gcps:
        add_gcp_to_bundle(ba, scene, gcps, c, len(subset), n_shots, set(range(n_shots)))
    if c["bundle_compensate_gps_bias"] and gcps:
        idx = determine_gcp_bias_parameters(scene, gcps, c)
        biases = scene.extras.get("biases", {})
        for k in range(len(scene.camera_projection)):
            ba.set_camera_bias(str(k), biases.get(str(k), Similarity()), idx)
    _configure(ba, c, n_shots)
    ba.set_linear_solver_type(determine_linear_solver(n_shots))
    t_setup = time.perf_counter()
    ba.run()
    t_run = time.perf_counter()
    written = bundle_to_map(ba, scene, not fix_cameras, point_ids=subset)
    t_down = time.perf_counter()
    s = ba.summary()
    return {"brief_report": ba.brief_report(), "irls_report": ba.irls_report(), "full_report": ba.full_report(),
            "is_solution_usable": bool(s["usable"]), "summary": s,
            "wall_times": {"grid": t_grid - t0, "setup": t_setup - t_grid, "run": t_run - t_setup,
                           "teardown": t_down - t_run},
            "num_images": n_shots, "num_points": int(len(subset)), "num_reprojections": int(len(keep)),
            "other_tracks": other, "reprojection": written}


def bundle_local_stochastic(scene: SceneArrays, central_shots: Sequence[int], config: Optional[dict] = None,
                            gcps: Sequence[GroundControlPoint] = (), grid_size: Optional[int] = None,
                            precision: str = "mixed") -> Tuple[np.ndarray, dict]:
    """BundleLocalStochastic (ba_helpers.cc:442-804) on the GPU adjuster:
    the neighbourhood of the central shots, the grid-selected tracks of its
    interior, cameras and rig cameras fixed, an instance free only when all
    its shots are interior; with GPS-bias compensation (when asked and
    control points exist) every camera's bias is optimised, starting from
    the scene's, and every other GPS-bearing instance joins as a fixed,
    observation-free anchor with its prior; up-vector priors on the
    interior; ground control points; then the moving instances, the points
    and the biases written back.  Returns the point indices and the
    report."""
    import time
    c = _config(config)
    t0 = time.perf_counter()
    cov = Covisibility.of(scene)
    interior, boundary = shot_neighborhood(cov, central_shots, int(c["local_bundle_radius"]),
                                           int(c["local_bundle_min_common_points"]), int(c["local_bundle_max_shots"]))
    grid = c["local_bundle_grid"] if grid_size is None else grid_size
    width, height = scene.extras.get("width"), scene.extras.get("height")
    if width and height and grid > 1:
        subset, other = select_tracks_grid(scene, cov, interior, grid, int(width), int(height))
    else:
        subset = np.unique(np.concatenate([cov.shot_points[s] for s in sorted(interior)])) if interior \
            else np.zeros(0, np.int64)
        other = np.zeros(0, np.int64)
    ba = pybundle.BundleAdjuster()
    ba.set_precision(precision)
    for k in range(len(scene.camera_projection)):
        m = int(scene.camera_projection[k])
        cam = Camera(m, scene.camera_values[k, : NUM_PARAMS[m]])
        ba.add_camera(str(k), cam, cam, True)
    compensate = bool(c["bundle_compensate_gps_bias"]) and len(gcps) > 0
    if compensate:
        idx = determine_gcp_bias_parameters(scene, gcps, c)
        biases = scene.extras.get("biases", {})
        for k in range(len(scene.camera_projection)):
            ba.set_camera_bias(str(k), biases.get(str(k), Similarity()), idx)
    use_gps = bool(c["bundle_use_gps"])
    shots = interior | boundary
    instances = {int(cov.shot_instance[s]) for s in shots}
    if compensate and use_gps and "gps" in scene.extras:
        instances |= set(cov.instance_shots)  # every GPS-bearing instance, as a fixed anchor
    fixed = {i for i in instances if any(s not in interior for s in cov.instance_shots[i])}
    ba.add_rig_camera("rig", Pose(), Pose(), True)
    moving = _add_scene_shots(ba, scene, cov, sorted(instances), fixed, use_gps, compensate)
    up = _up_vector(scene, gcps, c)
    if up is not None:
        for s in sorted(interior):
            ba.add_absolute_up_vector(str(s), up, 1e-3)
    ba.add_points(scene.points[subset])
    local = -np.ones(len(scene.points), np.int64)
    local[subset] = np.arange(len(subset))
    keep = np.nonzero(np.isin(np.asarray(scene.obs_point), subset) &
                      np.isin(np.asarray(scene.obs_shot), sorted(shots)))[0]
    shot_index = {s: ba.shot_index(str(s)) for s in shots}
    ba.add_point_projection_observations(np.array([shot_index[int(s)] for s in np.asarray(scene.obs_shot)[keep]],
                                                  np.int32),
                                         local[np.asarray(scene.obs_point)[keep]].astype(np.int32),
                                         np.asarray(scene.obs_xy)[keep], np.asarray(scene.obs_std)[keep])
    if c["bundle_use_gcp"] and gcps:
        add_gcp_to_bundle(ba, scene, gcps, c, len(subset), len(shots), shots)
    _configure(ba, c, len(shots))
    ba.set_linear_solver_type(determine_linear_solver(len(shots)))
    t_setup = time.perf_counter()
    ba.run()
    t_run = time.perf_counter()
    for i in moving:
        scene.rig_instance_poses[i] = ba.get_rig_instance_pose(str(i)).ba_data()
    pts = ba.get_points()[: len(subset)]
    scene.points[subset] = pts
    if compensate:
        out = scene.extras.setdefault("biases", {})
        for k in range(len(scene.camera_projection)):
            b = ba.get_bias(str(k))
            if not b.is_valid():
                raise RuntimeError(f"Bias {k} has either NaN or INF values.")
            out[str(k)] = b
    s = ba.summary()
    report = {"brief_report": ba.brief_report(), "full_report": ba.full_report(), "irls_report": ba.irls_report(),
              "is_solution_usable": bool(s["usable"]), "summary": s,
              "wall_times": {"setup": t_setup - t0, "run": t_run - t_setup},
              "num_images": len(interior), "num_interior_images": len(interior),
              "num_boundary_images": len(boundary),
              "num_other_images": len(scene.shot_camera) - len(interior) - len(boundary),
              "num_points": int(len(subset)), "num_reprojections": int(len(keep)), "other_tracks": other}
    return subset, report


__all__ = ["Covisibility", "DEFAULT_CONFIG", "GroundControlPoint", "LocalProblem", "add_gcp_to_bundle",
           "alignment_constraints", "are_points_collinear", "bundle_full", "bundle_local", "bundle_local_batch",
           "bundle_local_stochastic", "bundle_shot_poses", "bundle_stochastic", "bundle_to_map",
           "detect_alignment_constraints", "determine_gcp_bias_parameters", "determine_linear_solver",
           "direct_shot_neighbors", "local_problem", "select_tracks_grid", "shot_neighborhood", "shot_poses_problem",
           "stochastic_rounds", "stochastic_seeds", "triangulate_gcp"]
