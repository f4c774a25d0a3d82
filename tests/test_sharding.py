"""Tank sharding and data-parallel training: the host logic on CPU with two
gloo ranks, and on one GPU the sharded tanks against the unsharded batch."""
from __future__ import annotations

import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from computer_graphics_lab_00_gb300.sharding import (TankStats, data_parallel_step, partition_tanks, reduce_stats,
                                                     shard_loads)
from oracle import mlp_oracle as M


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _run_gloo(fn, world: int, *args):
    port = _free_port()
    ctx = mp.get_context("spawn")
    queue = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(fn, r, world, port, queue, args)) for r in range(world)]
    for p in procs:
        p.start()
    results = {}
    for _ in range(world):
        rank, value = queue.get(timeout=120)
        results[rank] = value
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    return [results[r] for r in range(world)]


def _worker(fn, rank, world, port, queue, args):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        queue.put((rank, fn(rank, world, *args)))
    finally:
        dist.destroy_process_group()


# -- partition ---------------------------------------------------------------------------------

@pytest.mark.parametrize("world", [1, 2, 3, 4, 8])
def test_partition_covers_every_tank_once_and_balances(world):
    rng = np.random.default_rng(world)
    counts = np.round(np.exp(rng.uniform(np.log(2048), np.log(65536), 256))).astype(int).tolist()
    shards = partition_tanks(counts, world)
    flat = sorted(t for s in shards for t in s)
    assert flat == list(range(256))
    loads = shard_loads(counts, shards)
    # Greedy LPT: no rank exceeds the mean by more than the largest tank.
    assert max(loads) - sum(counts) / world <= max(counts)
    assert partition_tanks(counts, world) == shards  # deterministic


def test_partition_edge_cases():
    assert partition_tanks([], 2) == [[], []]
    assert partition_tanks([5], 3) == [[0], [], []]
    assert partition_tanks([4, 4, 4, 4], 2) == [[0, 2], [1, 3]]
    with pytest.raises(ValueError):
        partition_tanks([1], 0)
    with pytest.raises(ValueError):
        partition_tanks([-1], 1)


# -- statistics reduction over gloo ------------------------------------------------------------

class _FakeStats:
    def __init__(self, particles, compression, density, ke, peak, nonfinite=0):
        self.particles = particles
        self.mean_compression = compression
        self.mean_density = density
        self.kinetic_energy = ke
        self.max_density = peak
        self.nonfinite = nonfinite


def _tank_stats(t):
    return _FakeStats(1000 + 37 * t, 0.01 * (t % 7), 990.0 + t, 0.5 * t, 1000.0 + 3 * t, t % 2)


def _reduce_worker(rank, world, counts):
    mine = partition_tanks(counts, world)[rank]
    return reduce_stats(TankStats.from_sph_stats([_tank_stats(t) for t in mine]))


def test_reduce_stats_over_two_gloo_ranks():
    counts = [1000 + 37 * t for t in range(9)]
    got = _run_gloo(_reduce_worker, 2, counts)
    want = reduce_stats(TankStats.from_sph_stats([_tank_stats(t) for t in range(9)]))
    for r in got:
        assert r["particles"] == want["particles"]
        assert r["nonfinite"] == want["nonfinite"]
        assert r["max_density"] == want["max_density"]
        for k in ("mean_compression", "mean_density", "kinetic_energy"):
            assert r[k] == pytest.approx(want[k], rel=1e-12)


# -- data-parallel Adam over gloo, with the oracle as the per-rank MLP -----------------------

def _case(n=256, seed=3):
    rng = np.random.default_rng(seed)
    params = np.zeros(M.PARAMS)
    params[M.W1:M.B1] = rng.normal(0, np.sqrt(2 / 32), M.HIDDEN * M.IN)
    params[M.W2:M.B2] = rng.normal(0, np.sqrt(2 / 128), M.HIDDEN * M.HIDDEN)
    params[M.W3:M.B3] = rng.normal(0, np.sqrt(2 / 128), M.OUT * M.HIDDEN)
    f = rng.normal(0, 1, (n, M.IN)).astype(np.float32)
    t = rng.normal(0, 1, (n, M.OUT)).astype(np.float32)
    mean = np.zeros(M.IN, np.float32)
    std = np.ones(M.IN, np.float32)
    scale = np.ones(M.OUT, np.float32)
    return params.astype(np.float32), f, t, mean, std, scale


def _train(rank, world, steps):
    params, f, t, mean, std, scale = _case()
    n = f.shape[0] // world
    mine = slice(rank * n, (rank + 1) * n)
    first = np.zeros(M.PARAMS, np.float32)
    second = np.zeros(M.PARAMS, np.float32)
    losses = []
    for step in range(1, steps + 1):
        def grads():
            loss, g = M.loss_and_grad(params, f[mine], t[mine], mean, std, scale)
            return loss, g.astype(np.float32)

        def apply(g, step=step):
            M.adam_step(params, g, first, second, step, 1e-3)

        losses.append(data_parallel_step(grads, apply))
    return params.copy(), losses


def test_data_parallel_adam_equals_single_process_full_batch():
    steps = 3
    (p0, l0), (p1, l1) = _run_gloo(_train, 2, steps)
    np.testing.assert_array_equal(p0, p1)  # every rank applies the same update
    assert l0 == l1
    # Same run on one process with the whole batch.
    params, f, t, mean, std, scale = _case()
    first = np.zeros(M.PARAMS, np.float32)
    second = np.zeros(M.PARAMS, np.float32)
    for step in range(1, steps + 1):
        loss, g = M.loss_and_grad(params, f, t, mean, std, scale)
        M.adam_step(params, g.astype(np.float32), first, second, step, 1e-3)
    # Averaging two half-batch means in FP32 differs from the full mean by rounding only.
    np.testing.assert_allclose(p0, params, rtol=0, atol=1e-6)


# -- sharded tanks on one GPU ------------------------------------------------------------------

@pytest.mark.gpu
def test_sharded_tanks_equal_the_unsharded_batch(native):
    """Tanks are independent: two shards stepped apart give every tank the
    bits the whole batch gives it, and the shard statistics sum to the
    batch's. (Both shards run on one GPU here, one after the other; no rank
    waits on another.)"""
    from computer_graphics_lab_00_gb300 import workloads as W
    from computer_graphics_lab_00_gb300.batch import BatchSolverGpu
    from computer_graphics_lab_00_gb300.sharding import ShardedBatch

    ts = W.batched_tanks(12, seed=5)
    whole = BatchSolverGpu(ts.params, ts.counts)
    for t in range(len(ts.counts)):
        whole.upload(t, *ts.initial_state(t))
    whole.run(ts.dt, 4)
    want = [whole.download(t) for t in range(len(ts.counts))]
    want_stats = reduce_stats(TankStats.from_sph_stats(whole.stats()))
    whole.close()

    parts = [ShardedBatch(ts, r, 2) for r in range(2)]
    for part in parts:
        part.run(ts.dt, 4)
        part.synchronize()
    seen = set()
    local = []
    for part in parts:
        for k, t in enumerate(part.tanks):
            pos, vel = part.solver.download(k)
            np.testing.assert_array_equal(pos, want[t][0])
            np.testing.assert_array_equal(vel, want[t][1])
            seen.add(t)
        local.append(part.local_stats())
        part.close()
    assert seen == set(range(len(ts.counts)))
    merged = TankStats()
    for s in local:
        merged.particles += s.particles
        merged.compression_sum += s.compression_sum
        merged.density_sum += s.density_sum
        merged.kinetic_energy += s.kinetic_energy
        merged.max_density = max(merged.max_density, s.max_density)
        merged.nonfinite += s.nonfinite
    got = reduce_stats(merged)
    assert got["particles"] == want_stats["particles"]
    assert got["max_density"] == want_stats["max_density"]
    assert got["mean_compression"] == pytest.approx(want_stats["mean_compression"], rel=1e-12)
    assert got["kinetic_energy"] == pytest.approx(want_stats["kinetic_energy"], rel=1e-12)


@pytest.mark.gpu
def test_apply_gradients_matches_train_step(native):
    """sph_mlp_apply_gradients with the gradient sph_mlp_gradients returned
    performs the same Adam step as sph_mlp_train_step."""
    from computer_graphics_lab_00_gb300.learned import MlpGpu

    rng = np.random.default_rng(4)
    f = torch.from_numpy(rng.normal(0, 1, (512, 32)).astype(np.float32)).cuda()
    t = torch.from_numpy(rng.normal(0, 1, (512, 3)).astype(np.float32)).cuda()
    torch.cuda.synchronize()
    with MlpGpu(seed=9) as a, MlpGpu(seed=9) as b:
        for _ in range(3):
            a.train_step(f.data_ptr(), t.data_ptr(), 512, 1e-3)
            _, g = b.gradients(f.data_ptr(), t.data_ptr(), 512)
            b.apply_gradients(g, 1e-3)
        np.testing.assert_array_equal(a.params(), b.params())
