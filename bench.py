#!/usr/bin/env python
"""Benchmark of the GB300 bundle adjuster.

Metric (one JSON line on rank 0):
  "BA time-to-converge (rel cost 1e-6) mixed vs FP64 GPU; Mobs/s residual+Jacobian"

* value -- residual + Jacobian evaluation throughput in Mobs/s (mixed
  precision: FP64 camera centring, FP32 residual/Jacobian records) over the
  whole workload with every input resident in HBM.  One step = one pass over
  all observations (per-shot pose precompute + per-observation record
  kernel).  Inputs (300+ MB) and records (1.5+ GB) exceed the 129 MB L2.
* e2e -- the same metric through the reference-facing C-ABI call
  gbba_evaluate_projections with host buffers: host->device copy of the
  scene, evaluation, device->host copy of the FP64 residual/Jacobian blocks.
* converge -- the other half of the metric: a full Levenberg-Marquardt solve
  in mixed precision and in plain FP64 on the same workload (added when the
  solver runs on the device).
* roofline -- of the record kernel: algorithmic bytes (observation inputs,
  points, records written) per launch / CUDA-event time of that launch.
* cpu_baseline -- the FP64 CPU oracle (a restatement of the reference's
  ReprojectionError2DAnalytic evaluation; Ceres/OpenSfM cannot be built on
  these machines) on a bounded sample, all host threads.

Usage:
  python bench.py [--gpus N] [--steps K] [--warmup W] [--workload aerial|street|ring]
  python bench.py --impl reference ...   (CPU reference arm)
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "BA time-to-converge (rel cost 1e-6) mixed vs FP64 GPU; Mobs/s residual+Jacobian"
UNIT = "Mobs/s"
CLOCK_WINDOW_S = 1.5


def make_workload(name: str, seed_offset: int = 0):
    from opensfm_gb300 import synthetic as syn
    if name == "aerial":
        scene = syn.aerial_scene(seed=3 + seed_offset)
        cfg = {"workload": "aerial nadir BA: 70x72=5040 perspective cameras, 2M terrain points, "
                           "~15M observations, GPS priors, UTM-scale coordinates",
               "n_shots": 5040}
    elif name == "aerial_small":
        scene = syn.aerial_scene(seed=3 + seed_offset, n_points=300_000)
        cfg = {"workload": "aerial nadir BA, profiling size: 5040 cameras, 300k points, ~2.2M observations",
               "n_shots": 5040}
    elif name == "street":
        scene = syn.street_scene(seed=7 + seed_offset)
        cfg = {"workload": "street BA: 500 Brown cameras (4 models), 200k points, ~1.4M observations, "
                           "2% outliers", "n_shots": 500}
    elif name == "ring":
        scene = syn.ring_scene(seed=42 + seed_offset)
        cfg = {"workload": "ring BA: 20 perspective cameras, 2k points, 12k observations", "n_shots": 20}
    else:
        raise SystemExit(f"unknown workload {name}")
    cfg.update(n_points=int(len(scene.points)), n_observations=int(scene.n_observations))
    return scene, cfg


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines: list[str] = []
        self._t = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except FileNotFoundError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        if self._t:
            self._t.join(timeout=2)

    def summary(self) -> dict:
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(smax)), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": d["hbm_gbs"], "bf16_tflops": d.get("bf16_tflops", 1900.0), "source": "measured"}
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "source": "fallback"}


def traffic_per_obs(kernel: str, workload: str = "aerial_small"):
    """DRAM bytes (read + write) per observation of a kernel, from the
    committed ncu summary of one launch (profiles/<kernel>_<workload>.md,
    line "DRAM bytes per observation (...): B").  Traffic grows with the
    observations processed, so the per-launch figure of the bench is this
    times its observation count."""
    import re
    p = ROOT / "profiles" / f"{kernel}_{workload}.md"
    if not p.exists():
        return None
    m = re.search(r"^DRAM bytes per observation[^:]*:\s*([0-9.]+)", p.read_text(), re.M)
    return float(m.group(1)) if m else None


def cpu_baseline(scene, target_s: float = 10.0) -> dict:
    """FP64 CPU oracle evaluation on a bounded sample, all host threads."""
    from oracle import oracle
    threads = os.cpu_count() or 1
    n = scene.n_observations
    probe = min(n, 200_000)
    sub = scene.subset_observations(np.arange(probe))
    oracle.evaluate_scene(sub, threads)  # warm
    t0 = time.perf_counter()
    oracle.evaluate_scene(sub, threads)
    rate = probe / max(time.perf_counter() - t0, 1e-9)
    m = int(min(n, max(probe, rate * target_s)))
    sub = scene.subset_observations(np.arange(m))
    # one timed pass over the sample, then whole passes up to about target_s
    t0 = time.perf_counter()
    oracle.evaluate_scene(sub, threads)
    one = time.perf_counter() - t0
    reps = max(1, int(round(target_s / max(one, 1e-9))))
    t0 = time.perf_counter()
    for _ in range(reps):
        oracle.evaluate_scene(sub, threads)
    dt = time.perf_counter() - t0
    return {"value": m * reps / dt / 1e6, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"first {m} of {n} observations x {reps} passes, FP64 residual+Jacobian blocks, "
                      f"{threads} threads, {dt:.1f} s"}


def fp64_eval_rate(scene, steps: int, warmup: int, stream) -> dict:
    """Device residual+Jacobian throughput with FP64 records (FP64
    arithmetic throughout), timed like the mixed passes: CUDA events on the
    launching stream around `steps` passes after `warmup` untimed ones."""
    import torch
    from opensfm_gb300 import _lib
    from opensfm_gb300.scene import Evaluator
    ev = Evaluator(scene, _lib.PRECISION_FP64)
    sh = stream.cuda_stream
    with torch.cuda.stream(stream):
        for _ in range(warmup):
            ev.run(sh)
        torch.cuda.synchronize()
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        for _ in range(steps):
            ev.run(sh)
        t1.record(stream)
        torch.cuda.synchronize()
    dt = t0.elapsed_time(t1) / 1e3
    ev.close()
    return {"value": scene.n_observations * steps / dt / 1e6, "unit": UNIT, "ms_per_step": dt / steps * 1e3,
            "dtype": "f64", "record_bytes_per_obs": None}


def headline(result: dict) -> dict:
    """Compact summary of both halves of the metric, printed as the last key
    of the line (so that a reader of the line's tail sees it): device and
    end-to-end evaluation rates, and the time-to-converge comparisons."""
    def r3(x):
        return None if x is None else float(f"{x:.4g}")
    h = {"eval_mixed_mobs": r3(result["value"]), "eval_fp64_mobs": r3(result["value_fp64"]["value"]),
         "e2e_mobs": r3(result["e2e"]["value"]), "roofline_frac": r3(result["roofline"]["frac"]),
         "cpu_port_mobs": r3(result.get("cpu_baseline", {}).get("value"))}
    c = result.get("converge")
    if c and not c.get("two_level_only"):
        h["c3_converge"] = {
            "mixed_s": r3(c["mixed"]["time_to_target_s"]), "fp64_s": r3(c["fp64"]["time_to_target_s"]),
            "speedup": r3(c["speedup_mixed_vs_fp64"]),
            "iters_mixed_fp64": [c["mixed"]["iterations_to_target"], c["fp64"]["iterations_to_target"]],
            "final_rel_mixed_vs_fp64": r3(c["mixed_final_rel_to_fp64"]),
            "point_rms_mm": r3(1e3 * c["mixed_vs_fp64_solution"]["point_rms_m"]),
            "centre_rms_mm": r3(1e3 * c["mixed_vs_fp64_solution"]["centre_rms_m"]),
            "rotation_rms_urad": r3(1e6 * c["mixed_vs_fp64_solution"]["rotation_rms_rad"])}
        tl = c.get("two_level")
        if tl:
            h["c3_converge_two_level"] = {
                "mixed_s": r3(tl["mixed"]["time_to_target_s"]), "fp64_s": r3(tl["fp64"]["time_to_target_s"]),
                "pcg_iterations_mixed_fp64": [tl["mixed"]["pcg_iterations"], tl["fp64"]["pcg_iterations"]],
                "final_rel_to_block_jacobi_fp64": [r3(tl["mixed"]["final_rel_to_block_jacobi_fp64"]),
                                                   r3(tl["fp64"]["final_rel_to_block_jacobi_fp64"])],
                "clusters": tl["mixed"]["clusters"], "probes": tl["mixed"]["probes"]}
    st = result.get("street")
    if st:
        h["c2_street"] = {
            "exact_fp64_s": r3(st["exact_fp64"]["time_to_target_s"]),
            "exact_iters": st["exact_fp64"]["iterations"],
            "exact_run_to_run_rel": r3(st["exact_run_to_run_rel"]),
            "pcg_mixed_s": r3(st["pcg_mixed"]["solve_s"]), "pcg_fp64_s": r3(st["pcg_fp64"]["solve_s"]),
            "pcg_speedup_mixed_vs_fp64": r3(st["pcg_speedup_mixed_vs_fp64"]),
            "pcg_final_rel_mixed_fp64": [r3(st["pcg_mixed"]["final_rel_to_exact"]),
                                         r3(st["pcg_fp64"]["final_rel_to_exact"])],
            "pcg_mixed_two_level_s": r3(st.get("pcg_mixed_two_level", {}).get("solve_s")),
            "pcg_mixed_two_level_final_rel": r3(st.get("pcg_mixed_two_level", {}).get("final_rel_to_exact")),
            "inlier_rms_px_exact": r3(st["exact_fp64"]["inlier_rms_px"])}
        if "oracle_rel" in st:
            oc = st["oracle_check"]
            h["c2_street"]["oracle_rel_fp64_mixed"] = [r3(st["oracle_rel"]["fp64"]), r3(st["oracle_rel"]["mixed"])]
            h["c2_street"]["small_cpu_vs_gpu_s"] = [r3(oc["oracle_seconds"]), r3(oc["fp64_gpu_seconds"])]
    cc = result.get("cpu_converge")
    if cc:
        h["c1_converge_cpu_vs_gpu_s"] = {"cpu_oracle": r3(cc["oracle"]["seconds"]), "gpu_fp64": r3(cc["fp64"]["seconds"]),
                                        "gpu_mixed": r3(cc["mixed"]["seconds"]),
                                        "rel_fp64_mixed": [r3(cc["fp64"]["rel_to_oracle"]),
                                                           r3(cc["mixed"]["rel_to_oracle"])]}
    b = result.get("batched_local_ba")
    if b:
        h["c4_batch"] = {"batch_s": r3(b.get("batch_s")), "one_at_a_time_s": r3(b.get("one_at_a_time_s")),
                         "speedup": r3(b.get("speedup")), "lm_iterations": b.get("batch_lm_iterations"),
                         "graph_launches": b.get("graph_launches"),
                         "solve_s_device_loop_vs_per_iteration": [r3(b.get("batch_solve_s")),
                                                                  r3(b.get("per_iteration_graph", {}).get("solve_s"))]}
        ex = b.get("exact_steps")
        if ex:
            h["c4_batch"]["exact_steps"] = {"problems": ex["n_problems"], "batch_s": r3(ex["batch_s"]),
                                            "single_dense_s": r3(ex["single_dense_one_at_a_time_s"]),
                                            "speedup": r3(ex["speedup"]),
                                            "converged_both": ex["converged_both"],
                                            "max_rel_cost_converged": r3(ex["max_rel_cost_batch_vs_single_converged"])}
    d = result.get("dense_rcs")
    if d and d.get("spd"):
        big = d["spd"][-1]
        h["dense_factor"] = {"n": big["n"], "ms": r3(big["factor_ms"]), "tflops": r3(big["factor_tflops"])}
    return h


def street_benchmark(n_shots: int = 500, n_points: int = 200_000, seed: int = 7, max_iterations: int = 200,
                     pcg_iterations: int = 100, outlier_ratio: float = 0.02, oracle: bool = True,
                     oracle_shots: int = 50, oracle_points: int = 20_000, oracle_iterations: int = 60) -> dict:
    """The medium terrestrial workload as specified: 500 Brown cameras
    sharing 4 camera models along a random-walk street, 200k points, ~1.4M
    observations, 2% outliers uniform over the image, soft-L1 loss (1 px).

    * exact: the linear solver the reference picks for this size
      (SPARSE_SCHUR above 200 shots, ba_helpers.cc:42-49), an exact solve of
      the reduced camera system.  Exact steps take FP64 records in either
      precision (mixed FP32 records perturb the nearly singular gauge
      directions that the exact solve then amplifies), so this run is the
      FP64 reference of the workload.  A second identical run measures the
      run-to-run spread: the atomics' summation order differs between runs,
      and with 2% uniform outliers under soft-L1 the trajectory is sensitive
      enough that two FP64 runs may stop in different nearby minima.
    * pcg: ITERATIVE_SCHUR in mixed precision (FP32 records and PCG, FP64
      cost/step) and in FP64, the precision comparison the metric asks for.
    Each run reports the time it takes to reach the exact run's final cost
    x (1 + 1e-6), when it does, and its final cost relative to it.

    Error against the FP64 CPU oracle: the oracle's LM (an unblocked
    single-threaded Cholesky of the reduced system) needs minutes for the
    full problem, so it solves a bounded street problem of the same kind
    (oracle_shots shots, oracle_points points, the same outlier ratio and
    loss) for oracle_iterations iterations, which the GPU solves in both
    precisions too; their final costs and RMS reprojection errors are
    compared with the oracle's, and the wall times give the CPU baseline of
    the solve."""
    from opensfm_gb300 import synthetic as syn
    from opensfm_gb300.pybundle import adjuster_from_scene
    loss = ("SoftLOneLoss", 1.0)
    kw = dict(loss=loss, irls="none", gps=False)

    def rms_px(e, inliers):
        # RMS reprojection error of the inliers (the 2% outliers, uniform over
        # the image, would dominate an RMS over every observation)
        e = e[inliers]
        return float(np.sqrt(np.mean(np.sum(e[:, :2] ** 2, axis=1))) * 1000.0)

    def run(scene, precision, solver, iterations, coarse_leaf=0):
        ba = adjuster_from_scene(scene, precision=precision, max_iterations=iterations, linear_solver=solver,
                                 coarse_leaf=coarse_leaf, **kw)
        t0 = time.perf_counter()
        ba.run()
        wall = time.perf_counter() - t0
        errs, _, _ = ba.projection_results()
        out = (ba.summary(), ba.trace(), errs, wall)
        del ba
        return out

    scene = syn.street_scene(n_shots=n_shots, n_points=n_points, seed=seed, outlier_ratio=outlier_ratio)
    out = {"n_shots": n_shots, "n_points": int(len(scene.points)), "n_observations": int(scene.n_observations),
           "outlier_ratio": outlier_ratio, "loss": list(loss), "max_iterations": max_iterations,
           "pcg_max_iterations": pcg_iterations}
    inl = ~scene.extras["outliers"]
    runs = {"exact_fp64": run(scene, "fp64", "SPARSE_SCHUR", max_iterations),
            "exact_fp64_repeat": run(scene, "fp64", "SPARSE_SCHUR", max_iterations),
            "pcg_mixed": run(scene, "mixed", "ITERATIVE_SCHUR", pcg_iterations),
            "pcg_fp64": run(scene, "fp64", "ITERATIVE_SCHUR", pcg_iterations),
            # the two-level PCG preconditioner (clusters of at most 16 shots)
            "pcg_mixed_two_level": run(scene, "mixed", "ITERATIVE_SCHUR", pcg_iterations, coarse_leaf=16)}
    c64 = runs["exact_fp64"][0]["final_cost"]
    target = c64 * (1.0 + 1e-6)
    for name, (s, tr, errs, wall) in runs.items():
        hit = np.nonzero(tr[:, 1] <= target)[0]
        out[name] = {"time_to_target_s": float(tr[hit[0], 2]) if len(hit) else None,
                     "iterations": s["iterations"], "final_cost": s["final_cost"],
                     "final_rel_to_exact": (s["final_cost"] - c64) / c64, "solve_s": s["seconds"],
                     "run_wall_s": wall, "unsuccessful_steps": int(s["unsuccessful_steps"]),
                     "dense_failures": int(s["linear_solver_failures"]),
                     "pcg_iterations": int(tr[:, 4].sum()), "inlier_rms_px": rms_px(errs, inl)}
    out["target_cost"] = target
    out["exact_run_to_run_rel"] = abs(runs["exact_fp64_repeat"][0]["final_cost"] - c64) / c64
    pm, pf = out["pcg_mixed"], out["pcg_fp64"]
    out["pcg_speedup_mixed_vs_fp64"] = (pf["solve_s"] / pm["solve_s"]) if pm["solve_s"] > 0 else None
    out["pcg_per_iteration_ms"] = {
        p: 1e3 * runs[f"pcg_{p}"][0]["linear_solver_seconds"] / max(1, out[f"pcg_{p}"]["pcg_iterations"])
        for p in ("mixed", "fp64")}
    if oracle:
        from oracle import oracle as orc
        small = syn.street_scene(n_shots=oracle_shots, n_points=oracle_points, seed=seed + 1,
                                 outlier_ratio=outlier_ratio)
        sinl = ~small.extras["outliers"]
        threads = os.cpu_count() or 1
        t0 = time.perf_counter()
        ref = orc.solve(small, loss=loss, irls="none", max_iterations=oracle_iterations, gps=False, threads=threads)
        cpu_s = time.perf_counter() - t0
        sruns = {p: run(small, p, "SPARSE_SCHUR", oracle_iterations) for p in ("fp64", "mixed")}
        out["oracle_check"] = {
            "n_shots": oracle_shots, "n_observations": int(small.n_observations),
            "iterations": oracle_iterations, "oracle_final_cost": ref["final_cost"],
            "oracle_iterations": ref["iterations"], "oracle_seconds": cpu_s, "oracle_threads": threads,
            "oracle_inlier_rms_px": rms_px(ref["errors"], sinl),
            **{f"{p}_rel_cost": abs(sruns[p][0]["final_cost"] - ref["final_cost"]) / ref["final_cost"]
               for p in ("fp64", "mixed")},
            **{f"{p}_inlier_rms_px_diff": abs(rms_px(sruns[p][2], sinl) - rms_px(ref["errors"], sinl))
               for p in ("fp64", "mixed")},
            **{f"{p}_gpu_seconds": sruns[p][3] for p in ("fp64", "mixed")}}
        out["oracle_rel"] = {p: out["oracle_check"][f"{p}_rel_cost"] for p in ("fp64", "mixed")}
    return out


def cpu_converge_baseline(max_iterations: int = 50) -> dict:
    """The solve on the host cores beside the GPU's, on the reference's own
    CPU-runnable configuration: the 20-camera ring (2,000 points, ~12k
    observations, Huber 1 px).  The FP64 CPU oracle (Ceres cannot be built
    on these machines) with every host thread, against the GPU solver in
    FP64 and mixed precision, each run to convergence; wall time from the
    call, setup included."""
    from oracle import oracle as orc
    from opensfm_gb300 import synthetic as syn
    from opensfm_gb300.pybundle import adjuster_from_scene
    scene = syn.ring_scene()
    threads = os.cpu_count() or 1
    loss = ("HuberLoss", 1.0)
    orc.solve(scene, loss=loss, irls="none", max_iterations=2, gps=False, threads=threads)  # warm
    t0 = time.perf_counter()
    ref = orc.solve(scene, loss=loss, irls="none", max_iterations=max_iterations, gps=False, threads=threads)
    cpu_s = time.perf_counter() - t0
    out = {"workload": "ring BA: 20 perspective cameras, 2k points, 12k observations, Huber 1 px",
           "oracle": {"seconds": cpu_s, "threads": threads, "iterations": ref["iterations"],
                      "final_cost": ref["final_cost"], "kind": "port"}}
    for precision in ("fp64", "mixed"):
        best = None
        for _ in range(3):
            ba = adjuster_from_scene(scene, precision=precision, loss=loss, irls="none",
                                     max_iterations=max_iterations, gps=False, linear_solver="SPARSE_SCHUR")
            t0 = time.perf_counter()
            ba.run()
            wall = time.perf_counter() - t0
            s = ba.summary()
            del ba
            if best is None or wall < best[0]:
                best = (wall, s)
        wall, s = best
        out[precision] = {"seconds": wall, "iterations": s["iterations"], "final_cost": s["final_cost"],
                          "rel_to_oracle": abs(s["final_cost"] - ref["final_cost"]) / ref["final_cost"]}
    out["speedup_fp64_vs_cpu"] = cpu_s / out["fp64"]["seconds"]
    return out


def converge_benchmark(scene, max_iterations: int, loss=("HuberLoss", 2.0), pcg_tolerance: float = 1e-3,
                       coarse_leaf: int = 32) -> dict:
    """Time to converge: FP64 and mixed-precision GPU solves of the same
    scene with a fixed objective (robust loss, IRLS off).  The FP64 solve's
    final cost C64 defines the target C64 * (1 + 1e-6); each solve reports
    the wall time (from the start of the solve, setup included) at which its
    cost first reaches the target.  With coarse_leaf > 0 both solves run
    again with the two-level PCG preconditioner, timed to the same target."""
    from opensfm_gb300.pybundle import adjuster_from_scene
    out = {"loss": list(loss), "irls": "none", "max_iterations": max_iterations, "pcg_tolerance": pcg_tolerance}
    runs = {}
    for precision in ("fp64", "mixed"):
        ba = adjuster_from_scene(scene, precision=precision, loss=loss, irls="none",
                                 max_iterations=max_iterations, pcg_tolerance=pcg_tolerance, gps=True)
        t0 = time.perf_counter()
        ba.run()
        wall = time.perf_counter() - t0
        s = ba.summary()
        # final poses [rx ry rz tx ty tz] and points, for the mixed-vs-FP64 errors
        poses = np.array([ba.get_rig_instance_pose(str(i)).ba_data() for i in range(len(scene.rig_instance_poses))])
        runs[precision] = {"trace": ba.trace(), "summary": s, "wall_s": wall, "points": ba.get_points(),
                           "poses": poses}
        del ba
    c64 = runs["fp64"]["summary"]["final_cost"]
    target = c64 * (1.0 + 1e-6)
    for precision, r in runs.items():
        tr = r["trace"]
        hit = np.nonzero(tr[:, 1] <= target)[0]
        s = r["summary"]
        out[precision] = {
            "time_to_target_s": float(tr[hit[0], 2]) if len(hit) else None,
            "iterations_to_target": int(tr[hit[0], 0]) if len(hit) else None,
            "final_cost": s["final_cost"], "initial_cost": s["initial_cost"], "iterations": s["iterations"],
            "solve_s": s["seconds"], "linear_solver_s": s["linear_solver_seconds"],
            "jacobian_s": s["jacobian_seconds"], "residual_s": s["residual_seconds"],
            "setup_s": s["setup_seconds"], "first_iterate_s": float(tr[0, 2]), "run_wall_s": r["wall_s"],
            "kernel_launches": s["kernel_launches"],
            "pcg_iterations": int(tr[:, 4].sum()),
        }
    out["target_cost"] = target
    # the same mixed solve with matrix-free passes (no stored Jacobian
    # records: what a problem too large for the records would run)
    ba = adjuster_from_scene(scene, precision="mixed", loss=loss, irls="none", max_iterations=max_iterations,
                             pcg_tolerance=pcg_tolerance, gps=True, matrix_free=1)
    ba.run()
    s, tr = ba.summary(), ba.trace()
    del ba
    hit = np.nonzero(tr[:, 1] <= target)[0]
    out["mixed_matrix_free"] = {
        "time_to_target_s": float(tr[hit[0], 2]) if len(hit) else None, "final_cost": s["final_cost"],
        "iterations": s["iterations"], "solve_s": s["seconds"], "linear_solver_s": s["linear_solver_seconds"],
        "pcg_iterations": int(tr[:, 4].sum()),
        "pcg_iteration_ms": 1e3 * s["linear_solver_seconds"] / max(1, int(tr[:, 4].sum())),
        "stored_pcg_iteration_ms": 1e3 * out["mixed"]["linear_solver_s"] / max(1, out["mixed"]["pcg_iterations"])}
    out["mixed_final_rel_to_fp64"] = abs(runs["mixed"]["summary"]["final_cost"] - c64) / c64
    # pose and point errors of the mixed solution against the FP64 one (the
    # GPS priors fix the gauge, so the solutions are directly comparable)
    dp = np.linalg.norm(runs["mixed"]["points"] - runs["fp64"]["points"], axis=1)
    dc = np.linalg.norm(runs["mixed"]["poses"][:, 3:] - runs["fp64"]["poses"][:, 3:], axis=1)
    dr = np.linalg.norm(runs["mixed"]["poses"][:, :3] - runs["fp64"]["poses"][:, :3], axis=1)
    out["mixed_vs_fp64_solution"] = {
        "point_rms_m": float(np.sqrt((dp ** 2).mean())), "point_max_m": float(dp.max()),
        "centre_rms_m": float(np.sqrt((dc ** 2).mean())), "centre_max_m": float(dc.max()),
        "rotation_rms_rad": float(np.sqrt((dr ** 2).mean())), "rotation_max_rad": float(dr.max())}
    tm, tf = out["mixed"]["time_to_target_s"], out["fp64"]["time_to_target_s"]
    out["speedup_mixed_vs_fp64"] = (tf / tm) if (tm and tf) else None
    # the same solves with the two-level PCG preconditioner (block-Jacobi plus
    # similarity modes over clusters of at most coarse_leaf rig instances),
    # timed to the same target (the block-Jacobi FP64 final cost)
    if coarse_leaf:
        two = {"coarse_leaf": coarse_leaf}
        for precision in ("fp64", "mixed"):
            ba = adjuster_from_scene(scene, precision=precision, loss=loss, irls="none",
                                     max_iterations=max_iterations, pcg_tolerance=pcg_tolerance, gps=True,
                                     coarse_leaf=coarse_leaf)
            ba.run()
            s, tr, info = ba.summary(), ba.trace(), ba.coarse_info()
            del ba
            hit = np.nonzero(tr[:, 1] <= target)[0]
            two[precision] = {
                "time_to_target_s": float(tr[hit[0], 2]) if len(hit) else None,
                "iterations_to_target": int(tr[hit[0], 0]) if len(hit) else None,
                "final_cost": s["final_cost"], "final_rel_to_block_jacobi_fp64": (s["final_cost"] - c64) / c64,
                "iterations": s["iterations"], "solve_s": s["seconds"], "setup_s": s["setup_seconds"],
                "linear_solver_s": s["linear_solver_seconds"], "pcg_iterations": int(tr[:, 4].sum()),
                "pcg_per_lm_iteration": tr[1:, 4].astype(int).tolist(), **info}
        t2m, t2f = two["mixed"]["time_to_target_s"], two["fp64"]["time_to_target_s"]
        two["speedup_mixed_vs_fp64"] = (t2f / t2m) if (t2m and t2f) else None
        two["speedup_vs_block_jacobi"] = {
            "mixed": (tm / t2m) if (tm and t2m) else None, "fp64": (tf / t2f) if (tf and t2f) else None}
        out["two_level"] = two
    return out


def two_level_run(scene, max_iterations: int, coarse_leaf: int, loss=("HuberLoss", 2.0),
                  pcg_tolerance: float = 1e-3) -> dict:
    """One mixed-precision solve of the converge configuration with the
    two-level PCG preconditioner, for launch lists (no target: the
    block-Jacobi solves that define it are not run)."""
    from opensfm_gb300.pybundle import adjuster_from_scene
    ba = adjuster_from_scene(scene, precision="mixed", loss=loss, irls="none", max_iterations=max_iterations,
                             pcg_tolerance=pcg_tolerance, gps=True, coarse_leaf=max(1, coarse_leaf))
    ba.run()
    s, tr = ba.summary(), ba.trace()
    return {"two_level_only": True, "final_cost": s["final_cost"], "iterations": s["iterations"],
            "solve_s": s["seconds"], "pcg_iterations": int(tr[:, 4].sum()),
            "pcg_per_lm_iteration": tr[1:, 4].astype(int).tolist(), **ba.coarse_info()}


def batch_benchmark(n_problems: int = 256, seed: int = 23, max_iterations: int = 50,
                    loss=("HuberLoss", 2.0), one_at_a_time: bool = True, exact_problems: int = 64) -> dict:
    """Batched local bundle adjustment: n_problems uneven problems (5-60
    shots, 500-20k points, 3k-150k observations, log-uniform; Brown, fisheye
    and spherical cameras with fixed intrinsics) solved by one batch
    (per-problem trust regions on the device, one LM iteration replayed as a
    CUDA graph, autotuned slot-kernel grid) against the same problems solved
    one at a time by the single-problem solver.  Mixed precision, PCG
    tolerance 1e-3, no IRLS.  Then exact steps (DENSE_SCHUR) on the first
    exact_problems problems: one batch against the single-problem dense
    solver one at a time."""
    from opensfm_gb300 import synthetic as syn
    from opensfm_gb300.pybundle import BundleBatch, adjuster_from_scene
    scenes = syn.local_ba_problems(n_problems, seed=seed)

    def adjusters():
        # the same linear solver as the batch (PCG on the implicit Schur product)
        return [adjuster_from_scene(s, precision="mixed", loss=loss, irls="none", gps=False, constant_cameras=True,
                                    max_iterations=max_iterations, pcg_tolerance=1e-3,
                                    linear_solver="ITERATIVE_SCHUR") for s in scenes]

    out = {"n_problems": n_problems, "n_observations": int(sum(s.n_observations for s in scenes)),
           "n_points": int(sum(len(s.points) for s in scenes)), "max_iterations": max_iterations,
           "loss": list(loss)}
    # warm-up batch (module loading, graph machinery)
    warm = adjusters()[:4]
    b = BundleBatch()
    for ba in warm:
        b.add(ba)
    b.run()
    bas = adjusters()
    b = BundleBatch()
    for ba in bas:
        b.add(ba)
    b.set_options(precision="mixed", max_iterations=max_iterations, pcg_iterations=100, pcg_tolerance=1e-3)
    t0 = time.perf_counter()
    b.run()
    batch_s = time.perf_counter() - t0
    s = b.summary()
    batch_costs = np.array([ba.summary()["final_cost"] for ba in bas])
    init_costs = np.array([ba.summary()["initial_cost"] for ba in bas])
    batch_conv = np.array([ba.summary()["iterations"] < max_iterations for ba in bas])
    out.update({"batch_s": batch_s, "batch_setup_s": s["setup_seconds"], "batch_solve_s": s["solve_seconds"],
                "batch_lm_iterations": s["lm_iterations"], "graph_nodes": s["graph_nodes"],
                "graph_launches": s["graph_launches"],
                "autotuned_grid": s["grid"], "converged_batch": int(batch_conv.sum()),
                "batch_mobs_per_s": out["n_observations"] / batch_s / 1e6})
    # the same batch with one graph launch per LM iteration and a host check
    # of the done count between them (the device-side loop removes those)
    bas1 = adjusters()
    b1 = BundleBatch()
    for ba in bas1:
        b1.add(ba)
    b1.set_options(precision="mixed", max_iterations=max_iterations, pcg_iterations=100, pcg_tolerance=1e-3,
                   use_graph=1)
    b1.run()
    s1 = b1.summary()
    out["per_iteration_graph"] = {"solve_s": s1["solve_seconds"], "lm_iterations": s1["lm_iterations"],
                                  "graph_launches": s1["graph_launches"]}
    if not one_at_a_time:
        return out
    # one at a time
    singles = adjusters()
    t0 = time.perf_counter()
    for ba in singles:
        ba.run()
    single_s = time.perf_counter() - t0
    single_costs = np.array([ba.summary()["final_cost"] for ba in singles])
    single_conv = np.array([ba.summary()["iterations"] < max_iterations for ba in singles])
    both = batch_conv & single_conv
    rel = np.abs(batch_costs - single_costs) / single_costs
    out.update({
        "batch_s": batch_s, "batch_setup_s": s["setup_seconds"], "batch_solve_s": s["solve_seconds"],
        "batch_lm_iterations": s["lm_iterations"], "graph_nodes": s["graph_nodes"], "autotuned_grid": s["grid"],
        "graph_launches": s["graph_launches"],
        "converged_batch": int(batch_conv.sum()), "converged_one_at_a_time": int(single_conv.sum()),
        "one_at_a_time_s": single_s, "speedup": single_s / batch_s,
        "batch_mobs_per_s": out["n_observations"] / batch_s / 1e6,
        "max_rel_cost_batch_vs_single_converged": float(rel[both].max()) if both.any() else None,
        "median_rel_cost_batch_vs_single_unconverged": float(np.median(rel[~both])) if (~both).any() else None,
        "mean_cost_reduction": float(np.mean(1.0 - batch_costs / init_costs)),
    })
    # exact steps (DENSE_SCHUR, the reference's linear solver for local
    # bundles): the first exact_problems problems as one batch against the
    # single-problem dense solver one at a time
    sub = scenes[:exact_problems]

    def exact_adjusters(single: bool):
        return [adjuster_from_scene(sc, precision="fp64", loss=loss, irls="none", gps=False, constant_cameras=True,
                                    max_iterations=max_iterations,
                                    linear_solver="DENSE_SCHUR" if single else "ITERATIVE_SCHUR") for sc in sub]
    be = exact_adjusters(False)
    b2 = BundleBatch()
    for ba in be:
        b2.add(ba)
    b2.set_options(precision="fp64", max_iterations=max_iterations, pcg_iterations=100, pcg_tolerance=1e-3)
    b2.set_linear_solver_type("DENSE_SCHUR")
    t0 = time.perf_counter()
    b2.run()
    exact_batch_s = time.perf_counter() - t0
    se = exact_adjusters(True)
    t0 = time.perf_counter()
    for ba in se:
        ba.run()
    exact_single_s = time.perf_counter() - t0
    eb = np.array([ba.summary()["final_cost"] for ba in be])
    es = np.array([ba.summary()["final_cost"] for ba in se])
    # problems that converge in both: the same exact trajectory; the others
    # stop at the iteration limit on chaotic non-monotonic paths
    conv = np.array([x.summary()["iterations"] < max_iterations and y.summary()["iterations"] < max_iterations
                     for x, y in zip(be, se)])
    rel = np.abs(eb - es) / es
    out["exact_steps"] = {
        "n_problems": len(sub), "n_observations": int(sum(sc.n_observations for sc in sub)),
        "batch_s": exact_batch_s, "batch_lm_iterations": b2.summary()["lm_iterations"],
        "single_dense_one_at_a_time_s": exact_single_s, "speedup": exact_single_s / exact_batch_s,
        "converged_both": int(conv.sum()),
        "max_rel_cost_batch_vs_single_converged": float(rel[conv].max()) if conv.any() else None,
        "median_rel_cost_unconverged": float(np.median(rel[~conv])) if (~conv).any() else None}
    return out


DENSE_STREET_RUNS = ("fp64:DENSE_SCHUR", "mixed:DENSE_SCHUR", "mixed:ITERATIVE_SCHUR", "fp64:ITERATIVE_SCHUR")


def dense_benchmark(sizes=(1024, 2048, 4096), street_shots: int = 500, street_points: int = 200_000,
                    max_iterations: int = 60, seed: int = 29, runs=DENSE_STREET_RUNS) -> dict:
    """Dense reduced-camera-system solver.

    (1) gbba_dense_spd_solve on seeded SPD matrices (condition 1e4): device
    time of the factorization (Jacobi scaling, FP32 conversion, tensor-core
    blocked Cholesky) and of the FP64 CG solve, and the factorization's
    algorithmic rate n^3/3 flop / s against the tensor roofline (TF32, taken
    as half the measured bf16 rate: the nominal dense TF32 / bf16 ratio).
    (2) The street workload (Brown cameras, soft-L1, outlier-free so that
    every run ends at the same minimum): the exact dense steps (DENSE_SCHUR)
    against PCG (ITERATIVE_SCHUR, tolerance 1e-3), FP64 and mixed; target =
    the FP64 dense final cost x (1 + 1e-6)."""
    from opensfm_gb300 import dense
    from opensfm_gb300 import synthetic as syn
    from opensfm_gb300.pybundle import adjuster_from_scene
    peaks = measured_peaks()
    tf32_peak = peaks["bf16_tflops"] / 2.0
    out = {"spd": []}
    rng = np.random.default_rng(seed)
    for n in sizes:
        q, _ = np.linalg.qr(rng.standard_normal((n, n)))
        a = (q * np.geomspace(1.0, 1e4, n)) @ q.T
        a = 0.5 * (a + a.T)
        b = rng.standard_normal(n)
        dense.spd_solve(a, b)  # warm-up (module load, kernel attributes)
        best = None
        for _ in range(3):
            x, st = dense.spd_solve(a, b)
            if best is None or st.factor_seconds < best.factor_seconds:
                best = st
        flops = n ** 3 / 3.0
        out["spd"].append({
            "n": n, "factor_ms": best.factor_seconds * 1e3, "solve_ms": best.solve_seconds * 1e3,
            "cg_iterations": best.refinements, "scaled_residual": best.rel_residual, "status": best.status,
            "factor_tflops": flops / best.factor_seconds / 1e12,
            "roofline": {"bound": "tensor", "achieved": flops / best.factor_seconds / 1e12, "peak": tf32_peak,
                         "unit": "TFLOP/s", "frac": flops / best.factor_seconds / 1e12 / tf32_peak,
                         "peak_source": "measured bf16 / 2 (nominal TF32 rate)"}})
    if street_shots <= 0:
        return out
    scene = syn.street_scene(n_shots=street_shots, n_points=street_points, seed=seed, outlier_ratio=0.0)
    loss = ("SoftLOneLoss", 1.0)
    out["street"] = {"n_shots": street_shots, "n_points": int(len(scene.points)),
                     "n_observations": int(scene.n_observations), "loss": list(loss),
                     "max_iterations": max_iterations}
    results = {}
    for spec in runs:
        precision, solver = spec.split(":")
        ba = adjuster_from_scene(scene, precision=precision, loss=loss, irls="none", gps=False,
                                 max_iterations=max_iterations, pcg_tolerance=1e-3, linear_solver=solver)
        ba.run()
        results[(precision, solver)] = (ba.summary(), ba.trace())
        del ba
    first = results[next(iter(results))][0]
    target = results.get(("fp64", "DENSE_SCHUR"), (first,))[0]["final_cost"] * (1.0 + 1e-6)
    out["street"]["target_cost"] = target
    for (precision, solver), (s, tr) in results.items():
        hit = np.nonzero(tr[:, 1] <= target)[0]
        out["street"][f"{precision}_{solver.lower()}"] = {
            "time_to_target_s": float(tr[hit[0], 2]) if len(hit) else None,
            "iterations": s["iterations"], "final_cost": s["final_cost"], "solve_s": s["seconds"],
            "linear_solver_s": s["linear_solver_seconds"], "linear_iterations": int(tr[:, 4].sum()),
            "setup_s": s["setup_seconds"], "dense_failures": int(s["linear_solver_failures"]),
            "unsuccessful_steps": int(s["unsuccessful_steps"])}
    return out


def outlier_benchmark(n_obs: int, seed: int = 31, reps: int = 3) -> dict:
    """Post-solve outlier selection (the observation test of
    sfm::BAHelpers::RemoveOutliers) on n_obs seeded 2D errors (1 mm Gaussian
    on a unit-width image plus 2% uniform outliers), IRLS weights and point
    indices (6 observations per point on average), FIXED and AUTO
    thresholds.  e2e: the C-ABI call on host buffers (errors upload
    included); device: the CUDA-event span from the inputs resident to the
    flags written.  Algorithmic bytes per observation: the 2D error (16 B),
    the weight (8 B), the point index (4 B) and the flag (1 B), plus one
    byte per point; the AUTO threshold reads the errors again for three
    exact radix selections (six 11-bit digit passes each).  CPU baseline:
    the oracle's numpy restatement on the same arrays."""
    from opensfm_gb300 import outliers
    from oracle import oracle
    rng = np.random.default_rng(seed)
    n_points = max(1, n_obs // 6)
    err = rng.normal(0.0, 1e-3, (n_obs, 3))
    bad = rng.random(n_obs) < 0.02
    err[bad, :2] = rng.uniform(-0.05, 0.05, (int(bad.sum()), 2))
    w = rng.uniform(0.3, 1.0, n_obs)
    pts = rng.integers(0, n_points, n_obs).astype(np.int32)
    peaks = measured_peaks()
    algo = 29.0 * n_obs + n_points
    out = {"n_observations": n_obs, "n_points": n_points, "algorithmic_bytes": int(algo)}
    for mode in ("FIXED", "AUTO"):
        outliers.find_outliers(err, w, pts, n_points, filter_type=mode)  # warm-up
        best, best_dev, st = None, None, {}
        for _ in range(reps):
            st = {}
            t0 = time.perf_counter()
            thr, flags, removed = outliers.find_outliers(err, w, pts, n_points, stats=st, filter_type=mode)
            dt = time.perf_counter() - t0
            best = dt if best is None else min(best, dt)
            best_dev = st["device_seconds"] if best_dev is None else min(best_dev, st["device_seconds"])
        t0 = time.perf_counter()
        rthr, rflags, rremoved = oracle.remove_outliers(err, w, pts, n_points, filter_type=mode)
        cpu = time.perf_counter() - t0
        achieved = algo / best_dev / 1e9
        out[mode.lower()] = {
            "e2e_ms": best * 1e3, "device_ms": best_dev * 1e3, "threshold": thr, "n_outliers": st["n_outliers"],
            "n_removed_points": st["n_removed_points"],
            "matches_oracle": bool(thr == rthr and np.array_equal(flags, rflags) and np.array_equal(removed, rremoved)),
            "cpu_baseline": {"seconds": cpu, "kind": "port", "cores": 1, "sample": "the same arrays (numpy)"},
            "e2e_speedup_vs_cpu": cpu / best,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                         "frac": achieved / peaks["hbm_gbs"], "peak_source": peaks["source"]}}
    return out


def covariance_benchmark(street_shots: int = 500, street_points: int = 200_000, seed: int = 29,
                         max_iterations: int = 60) -> dict:
    """Pose covariances (set_compute_covariances) on the street workload
    with GPS priors on every shot (5 cm noise and std: they fix the gauge,
    without which the reduced camera system is singular and the reference's
    default covariances are returned): the same FP64 dense solve with and
    without them; the difference is the covariance time (the undamped
    reduced camera system assembled and factored once, then 6 FP64 CG
    columns of its inverse per instance)."""
    from opensfm_gb300 import synthetic as syn
    from opensfm_gb300.pybundle import adjuster_from_scene
    scene = syn.street_scene(n_shots=street_shots, n_points=street_points, seed=seed, outlier_ratio=0.0)
    rng = np.random.default_rng(seed + 1)
    centres = scene.extras["true_poses"][:, 3:]
    scene.extras["gps"] = np.ascontiguousarray(centres + rng.normal(0.0, 0.05, centres.shape))
    scene.extras["gps_std"] = np.full(centres.shape, 0.05)
    times = {}
    valid = None
    for cov in (False, True):
        ba = adjuster_from_scene(scene, precision="fp64", loss=("SoftLOneLoss", 1.0), irls="none", gps=True,
                                 max_iterations=max_iterations, linear_solver="DENSE_SCHUR", covariances=cov)
        t0 = time.perf_counter()
        ba.run()
        times[cov] = time.perf_counter() - t0
        if cov:
            valid = bool(ba.get_covariance_estimation_valid())
        del ba
    return {"n_shots": street_shots, "n_instances": street_shots, "solve_s": times[False],
            "solve_with_covariances_s": times[True], "covariance_s": times[True] - times[False],
            "valid": valid}


def autograd_benchmark(n_obs: int = 4_000_000, steps: int = 5, seed: int = 17) -> dict:
    """Differentiable projection operator over n_obs observations: forward +
    backward (gradients for intrinsics, poses and points) for Brown and
    FISHEYE62 cameras, FP32 and FP64, with the Jacobian saved by the forward
    pass ("stored") or evaluated again in the backward pass ("recompute")."""
    import torch
    from opensfm_gb300 import autograd as ag
    from opensfm_gb300 import synthetic as syn
    from opensfm_gb300.scene import BROWN, FISHEYE62
    out = {"n_observations": n_obs, "steps": steps, "runs": []}
    for model, mname in ((BROWN, "brown"), (FISHEYE62, "fisheye62")):
        scene = syn.projection_scene(n_obs, model, seed=seed)
        for dtype, dname in ((torch.float32, "f32"), (torch.float64, "f64")):
            cams, poses, pts, obs = ag.observations_from_scene(scene, dtype=dtype)
            leaves = [t.requires_grad_(True) for t in (cams, poses, pts)]
            for recompute in (False, True):
                stream = torch.cuda.current_stream()
                for _ in range(2):  # warm-up
                    r = ag.project_residuals(*leaves, obs, recompute)
                    r.backward(torch.ones_like(r))
                torch.cuda.synchronize()
                torch.cuda.reset_peak_memory_stats()
                base = torch.cuda.memory_allocated()
                e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
                fwd = bwd = 0.0
                for _ in range(steps):
                    e0.record(stream)
                    r = ag.project_residuals(*leaves, obs, recompute)
                    e1.record(stream)
                    r.backward(torch.ones_like(r))
                    e2.record(stream)
                    torch.cuda.synchronize()
                    fwd += e0.elapsed_time(e1)
                    bwd += e1.elapsed_time(e2)
                del r
                out["runs"].append({"model": mname, "dtype": dname, "mode": "recompute" if recompute else "stored",
                                    "forward_ms": fwd / steps, "backward_ms": bwd / steps,
                                    "forward_backward_mobs_per_s": n_obs / ((fwd + bwd) / steps / 1e3) / 1e6,
                                    "peak_extra_bytes": int(torch.cuda.max_memory_allocated() - base)})
            for t in leaves:
                t.grad = None
    return out


def run_reference(args) -> None:
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    scene, cfg = make_workload(args.workload)
    from oracle import oracle
    threads = os.cpu_count() or 1
    n = scene.n_observations
    # bounded sample: about 2 s of CPU work per step
    probe = min(n, 200_000)
    sub = scene.subset_observations(np.arange(probe))
    t0 = time.perf_counter()
    oracle.evaluate_scene(sub, threads)
    rate = probe / max(time.perf_counter() - t0, 1e-9)
    m = int(min(n, max(probe, rate * 2.0)))
    sub = scene.subset_observations(np.arange(m))
    for _ in range(args.warmup):
        oracle.evaluate_scene(sub, threads)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        oracle.evaluate_scene(sub, threads)
    dt = time.perf_counter() - t0
    value = m * args.steps / dt / 1e6
    sample = f"first {m} of {n} observations per step, FP64 residual+Jacobian blocks, {threads} threads"
    out = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic", "config": cfg,
           "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
           "note": "CPU restatement of the reference's analytic residual/Jacobian evaluation "
                   "(Ceres 2.2 / Eigen are not installable here, so the reference itself cannot be built)"}
    print(json.dumps(out), flush=True)


def run_ours(args) -> None:
    import torch
    from opensfm_gb300 import _lib
    from opensfm_gb300.scene import Evaluator, alloc_outputs, output_struct

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    scene, cfg = make_workload(args.workload, seed_offset=rank)
    n_obs = scene.n_observations
    L = _lib.lib()
    stream = torch.cuda.Stream()
    sh = stream.cuda_stream

    ev = Evaluator(scene, _lib.PRECISION_MIXED)
    for _ in range(args.warmup):
        ev.run(sh)
    torch.cuda.synchronize()

    rec_bytes = ev.record_bytes
    in_bytes = n_obs * (8 + 4 + 4 + 4) + len(scene.points) * 32
    ev_start = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ev_mid = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ev_end = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]

    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        w0 = time.perf_counter()
        t_all0 = torch.cuda.Event(enable_timing=True)
        t_all1 = torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            t_all0.record(stream)
            for k in range(args.steps):
                ev_start[k].record(stream)
                ev.prepare(sh)
                ev_mid[k].record(stream)
                ev.records(sh)
                ev_end[k].record(stream)
            t_all1.record(stream)
        torch.cuda.synchronize()
        # The timed region is milliseconds long, shorter than the sampler's
        # 200 ms period: keep the same kernel loop running (untimed) until
        # the window holds several clock samples.
        clock_window = CLOCK_WINDOW_S
        with torch.cuda.stream(stream):
            while time.perf_counter() - w0 < clock_window:
                for _ in range(50):
                    ev.run(sh)
                torch.cuda.synchronize()
    if dist:
        dist.barrier()
    elapsed = t_all0.elapsed_time(t_all1) / 1e3
    if dist:
        t = torch.tensor([elapsed], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        elapsed = float(t.item())
    rec_ms = float(np.mean([ev_mid[k].elapsed_time(ev_end[k]) for k in range(args.steps)]))
    value = n_obs * args.steps * world / elapsed / 1e6
    # the same passes with FP64 records: the device rate at the arithmetic
    # width of the CPU reference arm
    ev.close()
    value_fp64 = fp64_eval_rate(scene, args.steps, args.warmup, stream)
    ev = Evaluator(scene, _lib.PRECISION_MIXED)

    # e2e: the one-shot host-buffer call
    nr, cmax = scene.layout()
    out = alloc_outputs(n_obs, nr, cmax)
    o = output_struct(out)
    s = scene.ctypes()
    import ctypes as C
    e2e_steps = 0 if args.no_e2e else max(3, min(10, args.steps))
    if e2e_steps:
        # warm-up calls as for the device-side steps: the first calls also
        # fault the output pages in (on GB300 + Grace the kernels write the
        # caller's pageable buffers directly)
        for _ in range(args.warmup):
            _lib.check(L.gbba_evaluate_projections(C.byref(s), _lib.PRECISION_MIXED, C.byref(o)))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        _lib.check(L.gbba_evaluate_projections(C.byref(s), _lib.PRECISION_MIXED, C.byref(o)))
    e2e_dt = (time.perf_counter() - t0) / max(e2e_steps, 1)
    h2d = sum(a.nbytes for a in (scene.camera_projection, scene.camera_values, scene.rig_instance_poses,
                                 scene.shot_rig_instance, scene.shot_camera, scene.shot_rig_camera,
                                 scene.points, scene.obs_shot, scene.obs_point, scene.obs_xy, scene.obs_std))
    d2h = sum(a.nbytes for a in (out.residuals, out.jac_camera, out.jac_instance, out.jac_rig_camera,
                                 out.jac_point))

    peaks = measured_peaks()
    achieved = (in_bytes + rec_bytes) / (rec_ms / 1e3) / 1e9
    tpo = traffic_per_obs("eval_records_kernel")
    result = None
    if rank == 0:
        result = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": elapsed / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
            "data": "synthetic (seeded generator, opensfm_gb300.synthetic)",
            "config": dict(cfg, precision="mixed: FP64 centring, FP32 records",
                           l2="inputs and records larger than L2 (no flush needed)",
                           parallelism=f"replicas x{world}"),
            "e2e": {"value": (n_obs / e2e_dt / 1e6) if e2e_steps else None, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h),
                    "path": "gbba_evaluate_projections: host (pageable) scene in, FP64 Jacobian blocks out to "
                            "host buffers; on GB300 + Grace the kernels read and write host memory directly "
                            "over NVLink-C2C, elsewhere the scene is uploaded and the blocks downloaded",
                    "warmup_calls": int(args.warmup) if e2e_steps else 0, "timed_calls": int(e2e_steps)},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                         "frac": achieved / peaks["hbm_gbs"],
                         "traffic": (tpo * n_obs if tpo else None),
                         "kernel": "eval_records_kernel", "algorithmic_bytes": int(in_bytes + rec_bytes),
                         "kernel_ms": rec_ms, "peak_source": peaks["source"]},
            "clocks": dict(clocks.summary(), window=f"timed region plus an untimed continuation of the same "
                                                    f"kernel loop, {CLOCK_WINDOW_S:.1f} s in all"),
            "gpu_launches": args.steps * ev.launches_per_run,
            "value_fp64": value_fp64,
        }
        if not args.no_cpu_baseline:
            result["cpu_baseline"] = cpu_baseline(scene)
        if not args.no_converge:
            ev.close()
            if args.two_level_only:
                result["converge"] = two_level_run(scene, args.converge_iterations, args.coarse_leaf)
            else:
                result["converge"] = converge_benchmark(scene, args.converge_iterations, coarse_leaf=args.coarse_leaf)
        if not args.no_autograd:
            ev.close()
            result["autograd"] = autograd_benchmark(n_obs=args.autograd_observations)
        if not args.no_batch:
            ev.close()
            result["batched_local_ba"] = batch_benchmark(n_problems=args.batch_problems,
                                                         one_at_a_time=not args.batch_only)
        if not args.no_dense:
            ev.close()
            result["dense_rcs"] = dense_benchmark(sizes=tuple(args.dense_sizes), street_shots=args.dense_street_shots,
                                                  street_points=args.dense_street_points,
                                                  runs=tuple(args.dense_street_runs))
        if not args.no_outliers:
            ev.close()
            result["outlier_selection"] = outlier_benchmark(args.outlier_observations or n_obs)
        if not args.no_covariance:
            ev.close()
            result["covariances"] = covariance_benchmark(street_shots=args.covariance_shots)
        if not args.no_cpu_converge:
            ev.close()
            result["cpu_converge"] = cpu_converge_baseline()
        if not args.no_street:
            ev.close()
            result["street"] = street_benchmark(n_shots=args.street_shots, n_points=args.street_points,
                                                max_iterations=args.street_iterations,
                                                pcg_iterations=max(1, args.street_iterations // 2),
                                                oracle=not args.no_street_oracle)
        result["headline"] = headline(result)
        print(json.dumps(result), flush=True)
    ev.close()
    if dist:
        dist.destroy_process_group()


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="aerial", choices=["aerial", "aerial_small", "street", "ring"])
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-converge", action="store_true")
    ap.add_argument("--converge-iterations", type=int, default=60)
    ap.add_argument("--coarse-leaf", type=int, default=32,
                    help="cluster size of the converge leg's two-level runs (0: block-Jacobi only)")
    ap.add_argument("--two-level-only", action="store_true",
                    help="converge leg: only the mixed two-level solve (for launch lists)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-autograd", action="store_true")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--batch-problems", type=int, default=256)
    ap.add_argument("--batch-only", action="store_true", help="skip the one-at-a-time comparison")
    ap.add_argument("--autograd-observations", type=int, default=4_000_000)
    ap.add_argument("--no-dense", action="store_true")
    ap.add_argument("--no-outliers", action="store_true")
    ap.add_argument("--outlier-observations", type=int, default=0, help="0: the workload's observation count")
    ap.add_argument("--no-covariance", action="store_true")
    ap.add_argument("--no-street", action="store_true", help="skip the street (500 Brown cameras) solves")
    ap.add_argument("--no-cpu-converge", action="store_true", help="skip the ring solve on the host cores")
    ap.add_argument("--pcg-host-loop", action="store_true",
                    help="launch the PCG kernels one by one instead of as one graph per solve (profilers see "
                         "kernels inside graphs with conditional nodes only as a whole)")
    ap.add_argument("--no-street-oracle", action="store_true", help="skip the street solve of the FP64 CPU oracle")
    ap.add_argument("--street-shots", type=int, default=500)
    ap.add_argument("--street-iterations", type=int, default=200,
                    help="LM iterations of the street solves (the PCG runs take half, at least 1)")
    ap.add_argument("--street-points", type=int, default=200_000)
    ap.add_argument("--covariance-shots", type=int, default=500)
    ap.add_argument("--dense-sizes", type=int, nargs="*", default=[1024, 2048, 4096])
    ap.add_argument("--dense-street-shots", type=int, default=500, help="0: skip the street solves")
    ap.add_argument("--dense-street-points", type=int, default=200_000)
    ap.add_argument("--dense-street-runs", nargs="*", default=list(DENSE_STREET_RUNS),
                    help="precision:LINEAR_SOLVER pairs of the street solves")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        if args.pcg_host_loop:
            import functools
            from opensfm_gb300 import pybundle
            pybundle.adjuster_from_scene = functools.partial(pybundle.adjuster_from_scene, pcg_graph=False)
        run_ours(args)


if __name__ == "__main__":
    main()
