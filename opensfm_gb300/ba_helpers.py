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
from .pygeometry import Camera, Pose
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


__all__ = ["Covisibility", "LocalProblem", "bundle_local", "bundle_local_batch", "bundle_shot_poses",
           "bundle_stochastic", "direct_shot_neighbors", "local_problem", "select_tracks_grid", "shot_neighborhood",
           "shot_poses_problem", "stochastic_rounds", "stochastic_seeds"]
