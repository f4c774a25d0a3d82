"""The fluid surface on the CPU: the marching-cubes case table the device
uses (generated from the face-contour rule) checked for the properties
tests/marching_cubes_test.cpp:121-228 checks, and equal to the reference's
table; the oracle's buildFluidField / marchFluidField against the reference
(where its tree is present), the golden vectors, a brute-force field
(marching_cubes_test.cpp:265-318) and a cut sphere (:230-263)."""
from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

from computer_graphics_lab_00_gb300 import workloads as W
from computer_graphics_lab_00_gb300.abi import SURFACE_VERTEX, SphParams

GOLDEN = Path(__file__).resolve().parent / "golden"

CORNERS = np.array([(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)], float)
EDGES = [(0, 1), (1, 2), (2, 3), (3, 0), (4, 5), (5, 6), (6, 7), (7, 4), (0, 4), (1, 5), (2, 6), (3, 7)]
FACE_CORNERS = [(0, 1, 2, 3), (4, 5, 6, 7), (0, 1, 5, 4), (3, 2, 6, 7), (0, 3, 7, 4), (1, 2, 6, 5)]
FACE_EDGES = [(0, 1, 2, 3), (4, 5, 6, 7), (0, 9, 4, 8), (2, 10, 6, 11), (3, 11, 7, 8), (1, 10, 5, 9)]


def load(name):
    data = dict(np.load(GOLDEN / f"{name}.npz"))
    return SphParams.from_buffer_copy(data.pop("params").tobytes()), data


@pytest.fixture(scope="module")
def table():
    from computer_graphics_lab_00_gb300.fluid import surface_table

    return surface_table()


def entries(table, code):
    row = table[code]
    n = 0
    while n < 16 and row[n] >= 0:
        n += 1
    return [int(e) for e in row[:n]]


def inside(code, corner):
    return (code >> corner) & 1 == 1


def active(code, edge):
    return inside(code, EDGES[edge][0]) != inside(code, EDGES[edge][1])


def test_table_equals_golden_and_oracle(table, oracle):
    _, g = load("surface_small")
    np.testing.assert_array_equal(table, g["mc_table"])
    np.testing.assert_array_equal(oracle.mc_table(), g["mc_table"])


def test_table_equals_reference(table, reference_available):
    if not reference_available:
        pytest.skip("reference tree absent; the golden table pins it")
    from oracle.bind import Reference

    np.testing.assert_array_equal(table, Reference().mc_table())


def test_table_shape_and_edges(table):
    for code in range(256):
        e = entries(table, code)
        assert len(e) % 3 == 0 and len(e) <= 15
        assert all(x < 0 for x in table[code][len(e):])
        used = set(e)
        assert all(active(code, x) for x in used)
        assert all(x in used for x in range(12) if active(code, x))
        for i in range(0, len(e), 3):
            assert len({e[i], e[i + 1], e[i + 2]}) == 3


def test_table_winding_points_outward(table):
    mid = lambda x: (CORNERS[EDGES[x][0]] + CORNERS[EDGES[x][1]]) * 0.5  # noqa: E731
    for code in range(1, 255):
        e = entries(table, code)
        any_out = False
        for i in range(0, len(e), 3):
            a, b, c = (mid(x) for x in e[i:i + 3])
            normal = np.cross(b - a, c - a)
            out = np.zeros(3)
            for x in e[i:i + 3]:
                p, q = EDGES[x]
                frm, to = (p, q) if inside(code, p) else (q, p)
                out += CORNERS[to] - CORNERS[frm]
            facing = float(normal @ out)
            assert facing >= -1e-6
            any_out = any_out or facing > 1e-6
        assert not e or any_out
        directed = set()
        for i in range(0, len(e), 3):
            for k in range(3):
                edge = (e[i + k], e[i + (k + 1) % 3])
                assert edge not in directed
                directed.add(edge)


def test_table_face_contours_depend_on_face_signs_only(table):
    """No cracks: two cells sharing a face see the same contour on it."""
    for face in range(6):
        expected = {}
        on_face = set(FACE_EDGES[face])
        for code in range(256):
            pattern = sum(1 << k for k in range(4) if inside(code, FACE_CORNERS[face][k]))
            e = entries(table, code)
            directed = {(e[i + k], e[i + (k + 1) % 3]) for i in range(0, len(e), 3) for k in range(3)}
            contour = {tuple(sorted(d)) for d in directed
                       if (d[1], d[0]) not in directed and d[0] in on_face and d[1] in on_face}
            assert expected.setdefault(pattern, contour) == contour


def test_oracle_matches_golden_surface(oracle):
    params, g = load("surface_small")
    field = oracle.surface_field(params, g["pos"], 24, threads=4)
    np.testing.assert_array_equal(field.view(np.uint32), g["field_24"].view(np.uint32))
    origin = np.array(params.container_min[:3], np.float32)
    cell = ((np.array(params.container_max[:3], np.float32) - origin) / np.float32(24)).astype(np.float32)
    full = oracle.march_field(field, 24, origin, cell, 0.5, 200000)
    np.testing.assert_array_equal(full.view(np.uint8).reshape(-1, 16), g["vertices_24"])
    short = oracle.march_field(field, 24, origin, cell, 0.5, 600)
    np.testing.assert_array_equal(short.view(np.uint8).reshape(-1, 16), g["vertices_24_cap600"])
    assert len(oracle.march_field(field, 24, origin, cell, 0.5, 2)) == 0


def test_oracle_matches_reference_surface(oracle, reference_available):
    if not reference_available:
        pytest.skip("reference tree absent; the golden vectors pin the oracle")
    from oracle.bind import Reference

    ref = Reference()
    case = W.dam_break_16k()
    pos, vel = case.initial_state()
    pos, _ = oracle.run_substeps(case.params, pos, vel, case.dt, 150, threads=8)
    origin = np.array(case.params.container_min[:3], np.float32)
    span = np.array(case.params.container_max[:3], np.float32) - origin
    for resolution in (16, 40, 64):
        f_o = oracle.surface_field(case.params, pos, resolution, threads=8)
        f_r = ref.surface_field(case.params, pos, resolution, threads=8)
        np.testing.assert_array_equal(f_o.view(np.uint32), f_r.view(np.uint32))
        cell = (span / np.float32(resolution)).astype(np.float32)
        for iso, capacity in ((0.5, 300000), (0.2, 300000), (1.5, 4500), (0.5, 3)):
            v_o = oracle.march_field(f_o, resolution, origin, cell, iso, capacity)
            v_r = ref.march_field(f_r, resolution, origin, cell, iso, capacity)
            np.testing.assert_array_equal(v_o.view(np.uint8), v_r.view(np.uint8))


def lattice_particles():
    """marching_cubes_test.cpp:268-286: a jittered lattice, 8 per cell, no
    bucket overflow."""
    seed = 12345
    out = []
    spacing = np.float32(0.1)

    def jitter():
        nonlocal seed
        seed = (seed * 1664525 + 1013904223) & 0xFFFFFFFF
        return (np.float32(seed >> 8) / np.float32(16777216.0) - np.float32(0.5)) * np.float32(0.04)

    z = np.float32(-0.95)
    while z < np.float32(0.95):
        y = np.float32(0.05)
        while y < np.float32(1.95):
            x = np.float32(-0.95)
            while x < np.float32(0.95):
                out.append((x + jitter(), y + jitter(), z + jitter(), 0.0))
                x = np.float32(x + spacing)
            y = np.float32(y + spacing)
        z = np.float32(z + spacing)
    return np.array(out, np.float32)


def lattice_params():
    p = W.make_params(container_min=(-1.0, 0.0, -1.0), container_max=(1.0, 2.0, 1.0), lattice=(8, 8, 8),
                      cell_count=4096, spacing=0.1, smoothing_radius=0.2)
    return p


def test_oracle_field_equals_brute_force(oracle):
    params = lattice_params()
    particles = lattice_particles()
    resolution = 20
    field = oracle.surface_field(params, particles, resolution, threads=4)
    serial = oracle.surface_field(params, particles, resolution, threads=1)
    np.testing.assert_array_equal(field, serial)
    samples = resolution + 1
    origin = np.array(params.container_min[:3], np.float32)
    cell = ((np.array(params.container_max[:3], np.float32) - origin) / np.float32(resolution)).astype(np.float32)
    r2 = np.float32(0.2) * np.float32(0.2)
    grid = field.reshape(samples, samples, samples)
    nonzero = 0
    for z in range(samples):
        for y in range(samples):
            for x in range(samples):
                if 0 in (x, y, z) or resolution in (x, y, z):
                    assert grid[z, y, x] == 0.0
                    continue
                point = origin + np.array([x, y, z], np.float32) * cell
                d2 = ((particles[:, :3] - point) ** 2).sum(1)
                near = d2 < r2
                brute = float(((1.0 - d2[near] / r2) ** 3).sum())
                assert abs(grid[z, y, x] - brute) < 1e-4
                nonzero += brute > 0
    assert nonzero > 0


def sphere_field(resolution=24, radius=0.6):
    samples = resolution + 1
    idx = np.arange(samples, dtype=np.float32)
    coord = idx / np.float32(resolution) * np.float32(2.0) - np.float32(1.0)
    z, y, x = np.meshgrid(coord, coord, coord, indexing="ij")
    return (np.float32(radius) - np.sqrt(x * x + y * y + z * z)).astype(np.float32).reshape(-1)


def test_oracle_cuts_a_sphere_outward(oracle):
    """marching_cubes_test.cpp:230-263: vertices near the radius, triangles
    facing out."""
    resolution = 24
    cell = np.float32(2.0) / np.float32(resolution)
    v = oracle.march_field(sphere_field(resolution), resolution, (-1.0, -1.0, -1.0), (cell, cell, cell), 0.0, 200000)
    assert len(v) > 0 and len(v) % 3 == 0
    p = v["position"].astype(np.float64)
    assert np.all(np.abs(np.linalg.norm(p, axis=1) - 0.6) < cell)
    a, b, c = p[0::3], p[1::3], p[2::3]
    normal = np.cross(b - a, c - a)
    assert np.all((normal * (a + b + c) / 3.0).sum(1) > 0.0)
    assert SURFACE_VERTEX.itemsize == 16
