"""Synthetic workload generators (CPU): determinism and the stated shapes."""
from __future__ import annotations

import numpy as np

from computer_graphics_lab_00_gb300 import workloads as W


def test_batched_tanks_shape():
    ts = W.batched_tanks()
    assert len(ts.counts) == 256
    assert min(ts.counts) >= 2048 and max(ts.counts) <= 65536
    for t, p in enumerate(ts.params):
        ext = [p.container_max[a] for a in range(3)]
        assert all(0.5 <= e <= 2.0 for e in ext)
        assert p.lattice[0] * p.lattice[1] * p.lattice[2] >= ts.counts[t]
        assert p.lattice[3] == W.cell_count_for(ts.counts[t])
        pos, _ = ts.initial_state(t)
        lo = np.array([p.container_min[a] + p.container_min[3] for a in range(3)], np.float32)
        hi = np.array([p.container_max[a] - p.container_min[3] for a in range(3)], np.float32)
        assert (pos[:, :3] >= lo).all() and (pos[:, :3] <= hi).all(), t


def test_generators_are_deterministic():
    a = W.batched_tanks(tanks=8, seed=3)
    b = W.batched_tanks(tanks=8, seed=3)
    assert a.counts == b.counts
    assert all(bytes(x) == bytes(y) for x, y in zip(a.params, b.params))
    pa, _ = a.initial_state(5)
    pb, _ = b.initial_state(5)
    assert np.array_equal(pa.view(np.uint32), pb.view(np.uint32))
    assert W.batched_tanks(tanks=8, seed=4).counts != a.counts


def test_dam_break_configs():
    c16 = W.dam_break_16k()
    assert c16.count == 16384 and c16.params.lattice[3] == 32768
    c1m = W.dam_break_1m()
    assert c1m.count == 1 << 20 and c1m.params.lattice[3] == 1 << 21
    pos, vel = c1m.initial_state()
    assert pos.shape == (1 << 20, 4) and not vel.any()
    assert np.abs(pos[:, :3] - W.emit_positions(c1m.params, c1m.count)[:, :3]).max() <= 1e-4 + 1e-7
