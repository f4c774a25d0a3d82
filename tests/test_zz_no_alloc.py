"""sph_grid_build_static: the grid build for callers that cannot allocate
device memory when they call it (a render loop under a fixed memory budget,
or a loop that cannot take cudaMalloc's implicit synchronisation). Its
scratch is a static device array inside the library, so this file checks,
through the C ABI, that two calls in a row — which reuse that array and see
the previous call's leftovers — give exactly the grid of the allocating path
(sph_grid_build + sph_grid_download), and that sizes past the array's limit
are refused. Bucket keys, counts and slot order are integer results, so the
comparison is exact, as in the other grid tests. Each case is also compared
directly with the CPU oracle's grid build, and the sizes at the edges of the
static scratch (a full 65,536 particles in 65,536 buckets, one bucket, two
buckets) are covered.

Collected last on purpose: it needs only the library and a GPU, and passes
both alone in a fresh process and after the rest of the suite.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

from computer_graphics_lab_00_gb300 import abi
from computer_graphics_lab_00_gb300 import workloads as W
from computer_graphics_lab_00_gb300.fluid import FluidSolverGpu

pytestmark = pytest.mark.gpu


def allocating_grid(params, pos):
    with FluidSolverGpu(params, pos.shape[0]) as solver:
        solver.upload(pos)
        solver.build_grid()
        return solver.grid()


def static_grid(native, params, pos, offset_bytes: int = 0):
    import torch

    n = pos.shape[0]
    cells = int(params.lattice[3])
    d_pos = torch.from_numpy(np.ascontiguousarray(pos)).cuda()
    if offset_bytes:
        # The same positions starting `offset_bytes` into a larger buffer.
        raw = torch.zeros(pos.nbytes + 64, dtype=torch.uint8, device="cuda")
        raw[offset_bytes:offset_bytes + pos.nbytes] = d_pos.view(torch.uint8).reshape(-1)
        d_pos = raw
    d_cell_of = torch.empty(max(n, 1), dtype=torch.int32, device="cuda")
    d_counts = torch.empty(cells, dtype=torch.int32, device="cuda")
    d_slots = torch.full((cells * 32,), -1, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    status = native.sph_grid_build_static(ctypes.byref(params), ctypes.c_void_p(d_pos.data_ptr() + offset_bytes), n,
                                          ctypes.c_void_p(d_cell_of.data_ptr()), ctypes.c_void_p(d_counts.data_ptr()),
                                          ctypes.c_void_p(d_slots.data_ptr()), None)
    assert status == abi.SPH_OK, native.sph_status_string(status)
    torch.cuda.synchronize()
    to_u32 = lambda t: t.cpu().numpy().view(np.uint32)  # noqa: E731
    return to_u32(d_cell_of)[:n], to_u32(d_counts), to_u32(d_slots)


def assert_same_grid(got, want):
    cell_of, counts, slots = got
    w_cell_of, w_counts, w_slots = want
    np.testing.assert_array_equal(cell_of, w_cell_of)
    np.testing.assert_array_equal(counts, w_counts)
    used = (np.arange(32)[None, :] < np.minimum(counts, 32)[:, None]).reshape(-1)
    np.testing.assert_array_equal(slots[used], w_slots[used])


def test_static_grid_matches_allocating_grid_on_consecutive_calls(native):
    dam = W.dam_break_16k()
    dam_pos, _ = dam.initial_state()
    # A crowded case with few buckets: collisions and buckets past 32 slots.
    crowd = W.make_params(container_min=(0.0, 0.0, 0.0), container_max=(0.5, 0.5, 0.5), lattice=(8, 8, 64),
                          cell_count=1024)
    crowd_pos, _ = W.jittered_block(crowd, 4000, seed=9)
    crowd_pos[:300, :3] = np.float32(0.201) + W.uniform01(5, np.arange(900)).reshape(300, 3) * np.float32(0.038)
    for params, pos in ((dam.params, dam_pos), (crowd, crowd_pos), (dam.params, dam_pos)):
        assert_same_grid(static_grid(native, params, pos), allocating_grid(params, pos))


def test_static_grid_matches_the_oracle(native, oracle):
    dam = W.dam_break_16k()
    pos, _ = dam.initial_state()
    for _ in range(2):
        assert_same_grid(static_grid(native, dam.params, pos), oracle.grid_build(dam.params, pos))


@pytest.mark.parametrize("cells", [1, 2, abi.SPH_STATIC_MAX_CELLS])
def test_static_grid_at_the_edges_of_its_scratch(native, oracle, cells):
    # The full particle count; one bucket (a 0-bit key sorted as 1 bit), two
    # buckets, and the most buckets (the largest digit histogram region).
    n = abi.SPH_STATIC_MAX_PARTICLES
    params = W.make_params(container_min=(0.0, 0.0, 0.0), container_max=(1.0, 1.0, 1.0), lattice=(64, 32, 32),
                           cell_count=cells)
    pos, _ = W.jittered_block(params, n, seed=cells)
    want = oracle.grid_build(params, pos)
    for _ in range(2):
        got = static_grid(native, params, pos)
        assert_same_grid(got, want)
        assert_same_grid(got, allocating_grid(params, pos))


def test_static_grid_refuses_misaligned_positions(native):
    import torch

    params = W.dam_break_16k().params
    buf = torch.zeros(4096, dtype=torch.float32, device="cuda")
    out = torch.zeros(int(params.lattice[3]) * 32, dtype=torch.int32, device="cuda")
    base = buf.data_ptr()
    status = native.sph_grid_build_static(ctypes.byref(params), ctypes.c_void_p(base + 4), 64,
                                          ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(out.data_ptr()),
                                          ctypes.c_void_p(out.data_ptr()), None)
    assert status == abi.SPH_ERR_INVALID_ARGUMENT
    # A 16-byte aligned start inside the same buffer is accepted.
    pos, _ = W.jittered_block(params, 64, seed=1)
    assert_same_grid(static_grid(native, params, pos, offset_bytes=16), allocating_grid(params, pos))


def test_static_grid_refuses_sizes_past_its_scratch(native):
    import torch

    params = W.dam_break_16k().params
    dummy = torch.zeros(16, dtype=torch.int32, device="cuda")
    ptr = ctypes.c_void_p(dummy.data_ptr())
    too_many = abi.SPH_STATIC_MAX_PARTICLES + 1
    assert native.sph_grid_build_static(ctypes.byref(params), ptr, too_many, ptr, ptr, ptr, None) == abi.SPH_ERR_CAPACITY
    big = params.copy()
    big.lattice[3] = abi.SPH_STATIC_MAX_CELLS * 2
    assert native.sph_grid_build_static(ctypes.byref(big), ptr, 16, ptr, ptr, ptr, None) == abi.SPH_ERR_CAPACITY
