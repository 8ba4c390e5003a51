"""Point-partitioned (sharded) solve: the host side, on CPU.

* The partition (gbba_get_shard_points): contiguous point ranges that cover
  every point once, with nearly equal observation counts, the same on every
  rank.
* The decomposition the sharded solver relies on, with two gloo ranks: each
  rank evaluates only the observations of its own points (FP64 oracle), sums
  its share of the camera-side gradient J_c^T r and of the cost, and the
  ranks reduce them through the library's torch.distributed all-reduce
  (pybundle.torch_allreduce, the callback gbba_set_shard takes).  The
  reduced sums equal the single-process sums over all observations.
The solve itself needs a GPU: tests/test_gpu_shard.py.
"""
import multiprocessing as mp
import os
import socket

import numpy as np
import pytest

from opensfm_gb300 import pybundle
from opensfm_gb300 import synthetic as syn


def _adjuster(scene):
    return pybundle.adjuster_from_scene(scene, precision="fp64", irls="none", gps=False, max_iterations=5)


def _noop(a, op):
    pass


@pytest.mark.parametrize("world", [2, 3, 5])
def test_partition_covers_points_once_and_balances_observations(world):
    scene = syn.street_scene(n_shots=40, n_points=3000, seed=3, outlier_ratio=0.0)
    ba = _adjuster(scene)
    ba.set_shard(0, world, _noop)
    ranges = [ba.shard_points(r) for r in range(world)]
    assert ranges[0][0] == 0 and ranges[-1][1] == len(scene.points)
    for (a0, b0), (a1, b1) in zip(ranges, ranges[1:]):
        assert b0 == a1 and a0 <= b0
    counts = np.bincount(scene.obs_point, minlength=len(scene.points))
    per_rank = np.array([counts[a:b].sum() for a, b in ranges])
    assert per_rank.sum() == scene.n_observations
    # each range ends at the first point past its share: off by less than one
    # track from an equal split
    assert np.abs(per_rank - scene.n_observations / world).max() <= counts.max()
    # every rank computes the same partition
    other = _adjuster(scene)
    other.set_shard(world - 1, world, _noop)
    assert [other.shard_points(r) for r in range(world)] == ranges


def test_shard_arguments_are_checked():
    ba = _adjuster(syn.ring_scene(n_points=50))
    with pytest.raises(Exception):
        ba.set_shard(2, 2, _noop)
    with pytest.raises(ValueError):
        ba.set_shard(0, 2, None)
    ba.set_shard(0, 1)
    assert ba.shard_points(0) == (0, 50)


def _gradient_and_cost(scene, obs_idx):
    """Camera-side gradient (instance blocks, 6 per instance) and cost of
    the observations obs_idx, from the FP64 oracle."""
    from oracle import oracle
    sub = scene.subset_observations(obs_idx)
    res, jc, ji, jr, jp = oracle.evaluate_scene(sub, threads=1)
    g = np.zeros((len(scene.rig_instance_poses), 6))
    inst = sub.shot_rig_instance[sub.obs_shot]
    np.add.at(g, inst, np.einsum("nr,nrk->nk", res, ji))
    return g, 0.5 * float((res ** 2).sum())


def _rank_main(rank, world, port, q):
    try:
        import torch.distributed as dist
        from datetime import timedelta
        os.environ["MASTER_ADDR"] = "127.0.0.1"
        os.environ["MASTER_PORT"] = str(port)
        dist.init_process_group("gloo", rank=rank, world_size=world, timeout=timedelta(seconds=60))
        scene = syn.street_scene(n_shots=30, n_points=2000, seed=5, outlier_ratio=0.0)
        ba = _adjuster(scene)
        allreduce = pybundle.torch_allreduce()
        ba.set_shard(rank, world, allreduce)
        a, b = ba.shard_points(rank)
        mine = np.nonzero((scene.obs_point >= a) & (scene.obs_point < b))[0]
        g, c = _gradient_and_cost(scene, mine)
        buf = np.concatenate([g.reshape(-1), [c]])
        allreduce(buf, pybundle.REDUCE_SUM)
        mx = np.array([float(rank)])
        allreduce(mx, pybundle.REDUCE_MAX)
        dist.destroy_process_group()
        q.put((rank, buf, float(mx[0]), len(mine)))
    except Exception as e:  # pragma: no cover - reported to the parent
        q.put((rank, repr(e), None, None))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_ranks_reduce_to_the_full_gradient_and_cost():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = {}
    try:
        for _ in range(world):
            rank, buf, mx, n = q.get(timeout=180)
            assert not isinstance(buf, str), buf
            out[rank] = (buf, mx, n)
    finally:
        for p in procs:
            p.join(timeout=30)
            if p.is_alive():
                p.terminate()
    scene = syn.street_scene(n_shots=30, n_points=2000, seed=5, outlier_ratio=0.0)
    g, c = _gradient_and_cost(scene, np.arange(scene.n_observations))
    full = np.concatenate([g.reshape(-1), [c]])
    assert out[0][2] + out[1][2] == scene.n_observations and min(out[0][2], out[1][2]) > 0
    for rank in range(world):
        buf, mx, _ = out[rank]
        assert mx == world - 1
        scale = np.abs(full).max()
        assert np.abs(buf - full).max() <= 1e-12 * scale
    # both ranks hold bit-identical reduced values
    np.testing.assert_array_equal(out[0][0], out[1][0])
