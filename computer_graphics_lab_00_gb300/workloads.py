"""Seeded synthetic workloads for the SPH step.

No public dataset exists for this path, so every case is generated here:

* the reference's emit lattice (src/physics/fluid_sph.cpp:138-154) placed as
  a block whose lower corner sits one spacing inside the container, then
* a per-axis uniform jitter of +-1e-4 m drawn from splitmix64
  (the mixer of src/gfx/neural_math.cpp:18-24) keyed by (seed, 3*i + axis),
  using its top 24 bits as a uniform in [0, 1).

All float arithmetic is numpy float32, one rounding per operation, in the
order the reference writes it, so the same case is bit-identical on x86-64
and aarch64 hosts.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from .abi import SphParams

GOLDEN = np.uint64(0x9E3779B97F4A7C15)
MIX1 = np.uint64(0xBF58476D1CE4E5B9)
MIX2 = np.uint64(0x94D049BB133111EB)


def splitmix64(values: np.ndarray) -> np.ndarray:
    """splitmix64 finaliser over a uint64 array (wrapping arithmetic)."""
    v = np.asarray(values, dtype=np.uint64).copy()
    with np.errstate(over="ignore"):
        v += GOLDEN
        v = (v ^ (v >> np.uint64(30))) * MIX1
        v = (v ^ (v >> np.uint64(27))) * MIX2
    return v ^ (v >> np.uint64(31))


def uniform01(seed: int, index: np.ndarray) -> np.ndarray:
    """[0, 1) float32 from the top 24 bits of splitmix64(seed * golden + index)."""
    with np.errstate(over="ignore"):
        key = np.uint64(seed) * GOLDEN + np.asarray(index, dtype=np.uint64)
    bits = splitmix64(key) >> np.uint64(40)
    return bits.astype(np.float32) * np.float32(1.0 / 16777216.0)


def bit_ceil(x: int) -> int:
    return 1 if x <= 1 else 1 << (int(x) - 1).bit_length()


def cell_count_for(particles: int) -> int:
    """gfx::cellCountFor (src/gfx/fluid.cpp:50-52)."""
    return min(max(bit_ceil(max(particles, 1) * 2), 1024), 65536)


def cell_count_uncapped(particles: int) -> int:
    """cellCountFor without the 65536 ceiling (tanks beyond the reference's cap)."""
    return max(bit_ceil(max(particles, 1) * 2), 1024)


def translation(t) -> list[float]:
    """Column-major mat4 of a translation (glm::translate(mat4{1}, t))."""
    m = [0.0] * 16
    m[0] = m[5] = m[10] = m[15] = 1.0
    m[12], m[13], m[14] = float(t[0]), float(t[1]), float(t[2])
    return m


def make_params(
    *,
    container_min,
    container_max,
    lattice,
    cell_count: int,
    spacing: float = 0.02,
    smoothing_radius: float = 0.04,
    rest_density: float = 1000.0,
    stiffness: float = 50.0,
    viscosity: float = 0.5,
    gravity=(0.0, -9.81, 0.0),
    emitter_world=None,
    restitution: float = 0.3,
) -> SphParams:
    """A parameter block following deriveFluidParams (fluid_sph.cpp:65-100)."""
    f32 = np.float32
    s = f32(spacing)
    p = SphParams()
    if emitter_world is None:
        # Block whose lower corner is one spacing inside container_min.
        centre = [
            f32(container_min[a]) + s + f32(lattice[a] - 1) * s * f32(0.5) for a in range(3)
        ]
        emitter_world = translation(centre)
    for k in range(16):
        p.emitter_world[k] = float(f32(emitter_world[k]))
    for a in range(3):
        p.emitter_half_extents[a] = float(f32(lattice[a]) * s * f32(0.5))
        p.container_min[a] = float(container_min[a])
        p.container_max[a] = float(container_max[a])
        p.gravity[a] = float(gravity[a])
        p.lattice[a] = int(lattice[a])
    p.emitter_half_extents[3] = float(s)
    p.container_min[3] = float(s * f32(0.5))
    p.container_max[3] = float(f32(restitution))
    rho0 = f32(rest_density)
    p.gravity[3] = float(rho0 * s * s * s)
    p.smoothing_radius = float(max(f32(smoothing_radius), s))
    p.rest_density = float(rho0)
    p.stiffness = float(stiffness)
    p.viscosity = float(viscosity)
    p.lattice[3] = int(cell_count)
    return p


def emit_positions(params: SphParams, count: int) -> np.ndarray:
    """FluidSolver::emit lattice positions (N, 4) float32, w = rest density."""
    f32 = np.float32
    cx, cy, cz = (max(int(params.lattice[a]), 1) for a in range(3))
    s = f32(params.emitter_half_extents[3])
    i = np.arange(count, dtype=np.uint64)
    index = [i % np.uint64(cx), (i // np.uint64(cx)) % np.uint64(cy), i // np.uint64(cx * cy)]
    counts = (cx, cy, cz)
    local = []
    for a in range(3):
        extent = f32(counts[a] - 1) * s * f32(0.5)
        local.append(index[a].astype(np.float32) * s - extent)
    m = np.array(params.emitter_world[:], dtype=np.float32).reshape(4, 4)  # m[col][row]
    out = np.empty((count, 4), dtype=np.float32)
    one = f32(1.0)
    for r in range(3):
        add0 = m[0, r] * local[0] + m[1, r] * local[1]
        add1 = m[2, r] * local[2] + m[3, r] * one
        out[:, r] = add0 + add1
    out[:, 3] = f32(params.rest_density)
    return out


def jitter(count: int, seed: int, amplitude: float = 1e-4) -> np.ndarray:
    """(N, 3) float32 uniform in [-amplitude, +amplitude) from splitmix64(seed, 3i+axis)."""
    idx = np.arange(3 * count, dtype=np.uint64)
    u = uniform01(seed, idx).reshape(count, 3)
    return (u - np.float32(0.5)) * np.float32(2.0 * amplitude)


def jittered_block(params: SphParams, count: int, seed: int = 0, amplitude: float = 1e-4):
    """Positions (N,4) and zero velocities (N,4) of a jittered emit lattice."""
    pos = emit_positions(params, count)
    pos[:, :3] += jitter(count, seed, amplitude)
    vel = np.zeros((count, 4), dtype=np.float32)
    return pos, vel


@dataclass
class Case:
    """One single-tank workload: constants, particle count, step size and length."""

    name: str
    params: SphParams
    count: int
    dt: float
    steps: int
    seed: int = 0
    notes: str = ""
    extra: dict = field(default_factory=dict)

    def initial_state(self):
        return jittered_block(self.params, self.count, self.seed)


def dam_break_16k(seed: int = 0) -> Case:
    """Dam break, 16,384 particles in a 1 m box at s = 0.02, h = 0.04, dt = 1/600.

    The stated 0.32 x 0.64 x 0.32 m block holds 8,192 particles; the count is
    authoritative, so the reference's overflow rule (extra layers stack along
    z, fluid_sph.h:59) gives a 16 x 32 x 32 lattice.
    """
    n = 16384
    params = make_params(
        container_min=(0.0, 0.0, 0.0),
        container_max=(1.0, 1.0, 1.0),
        lattice=(16, 32, 32),
        cell_count=cell_count_for(n),
    )
    return Case("dam_break_16k", params, n, 1.0 / 600.0, 600, seed,
                "lattice 16x32x32 at 0.02 m, box [0,1]^3, C=32768")


def dam_break_1m(seed: int = 0) -> Case:
    """Dam break, 1,048,576 particles in a 4 x 2 x 2 m box at s = 0.02, h = 0.04.

    The stated 1.28 x 1.28 x 0.64 m block holds 131,072 particles; keeping the
    spacing and the count gives a 192 x 64 x 86 lattice (last z layer
    partial). The bucket count is bit_ceil(2N) = 2^21 without the
    reference's 65,536 ceiling, which would overflow the 32-slot buckets.
    """
    n = 1 << 20
    params = make_params(
        container_min=(0.0, 0.0, 0.0),
        container_max=(4.0, 2.0, 2.0),
        lattice=(192, 64, 86),
        cell_count=cell_count_uncapped(n),
    )
    return Case("dam_break_1m", params, n, 1.0 / 600.0, 1000, seed,
                "lattice 192x64x86 at 0.02 m, box 4x2x2 m, C=2^21")


def reference_test_scene(count: int = 1024, cell_count: int = 1024) -> SphParams:
    """The scene of the reference's fluid test (tests/fluid_test.cpp:19-32):
    scene::Fluid defaults, emitter at (0, 1, 0)."""
    f32 = np.float32
    r = f32(0.025)
    spacing = r * f32(2.0)
    half = f32(0.5)
    along = max(1, int(math.floor(float(half * f32(2.0) / spacing))))
    nz = max(1, (count + along * along - 1) // (along * along))
    return make_params(
        container_min=(-1.0, 0.0, -1.0),
        container_max=(1.0, 2.0, 1.0),
        lattice=(along, along, nz),
        cell_count=cell_count,
        spacing=float(spacing),
        smoothing_radius=0.1,
        emitter_world=translation((0.0, 1.0, 0.0)),
    )


# -- shape colliders and force fields (scene::ColliderShape, scene::ForceFieldType) ---------------

SPHERE, BOX, PLANE, CYLINDER, CAPSULE, MESH = range(6)
WIND, VORTEX, POINT = range(3)


def pose(position, axis_angle=None) -> np.ndarray:
    """Column-major float32 mat4 of a rotation (axis, angle in radians) then
    a translation: the world matrix of a collider."""
    m = np.eye(4, dtype=np.float64)
    if axis_angle is not None:
        axis = np.asarray(axis_angle[0], np.float64)
        axis = axis / np.linalg.norm(axis)
        c, s_ = math.cos(axis_angle[1]), math.sin(axis_angle[1])
        x, y, z = axis
        m[:3, :3] = [[c + x * x * (1 - c), x * y * (1 - c) - z * s_, x * z * (1 - c) + y * s_],
                     [y * x * (1 - c) + z * s_, c + y * y * (1 - c), y * z * (1 - c) - x * s_],
                     [z * x * (1 - c) - y * s_, z * y * (1 - c) + x * s_, c + z * z * (1 - c)]]
    m[:3, 3] = position
    return m.astype(np.float32)


def add_collider(params: SphParams, shape: int, world: np.ndarray, half_extents=(0.0, 0.0, 0.0),
                 radius: float = 0.0) -> None:
    """Appends a shape collider (gfx::GpuFluidCollider layout: world and
    inverse-world matrices, half extents, radius; y of the half extents is
    the half height of a cylinder or capsule)."""
    from .abi import SPH_MAX_COLLIDERS

    k = params.collider_count
    if k >= SPH_MAX_COLLIDERS:
        raise ValueError("at most 8 colliders")
    c = params.colliders[k]
    w = np.asarray(world, np.float32)
    inv = np.linalg.inv(w.astype(np.float64)).astype(np.float32)
    for col in range(4):
        for r in range(4):
            c.world[col * 4 + r] = float(w[r, col])
            c.inverse_world[col * 4 + r] = float(inv[r, col])
    for a in range(3):
        c.data0[a] = float(half_extents[a])
    c.data0[3] = float(radius)
    c.type = int(shape)
    params.collider_count = k + 1


def add_force_field(params: SphParams, kind: int, position, axis, strength: float, radius: float = 0.0,
                    falloff: float = 1.0) -> None:
    """Appends a force field (physics::ForceFieldSample in world space)."""
    from .abi import SPH_MAX_FORCE_FIELDS

    k = params.field_count
    if k >= SPH_MAX_FORCE_FIELDS:
        raise ValueError("at most 8 force fields")
    f = params.fields[k]
    for a in range(3):
        f.position_radius[a] = float(position[a])
        f.axis_strength[a] = float(axis[a])
    f.position_radius[3] = float(radius)
    f.axis_strength[3] = float(strength)
    f.falloff = float(falloff)
    f.type = int(kind)
    params.field_count = k + 1


def obstacle_course(seed: int = 0, count: int = 16384) -> Case:
    """The 16k dam break with one collider of every shape in its path and
    three force fields: a tilted plane ramp, a rotated box, a sphere, an
    upright cylinder and a lying capsule; a bounded wind, an unbounded vortex
    about y and a bounded point attractor. Falloffs are 1, where the
    reference's powf is exact."""
    case = dam_break_16k(seed)
    p = case.params
    add_collider(p, PLANE, pose((0.55, 0.05, 0.35), ((0.0, 0.0, 1.0), 0.35)))
    add_collider(p, BOX, pose((0.55, 0.12, 0.7), ((0.3, 1.0, 0.2), 0.6)), half_extents=(0.08, 0.1, 0.06))
    add_collider(p, SPHERE, pose((0.3, 0.1, 0.2)), radius=0.09)
    add_collider(p, CYLINDER, pose((0.8, 0.15, 0.5)), half_extents=(0.0, 0.15, 0.0), radius=0.07)
    add_collider(p, CAPSULE, pose((0.45, 0.08, 0.5), ((1.0, 0.0, 0.0), 1.5707964)), half_extents=(0.0, 0.12, 0.0),
                 radius=0.05)
    add_force_field(p, WIND, (0.5, 0.3, 0.5), (1.0, 0.0, 0.0), 3.0, radius=0.6, falloff=1.0)
    add_force_field(p, VORTEX, (0.5, 0.0, 0.5), (0.0, 1.0, 0.0), 4.0, radius=0.0)
    add_force_field(p, POINT, (0.7, 0.4, 0.5), (0.0, 0.0, 0.0), 5.0, radius=0.5, falloff=1.0)
    return Case("obstacle_course_16k", p, case.count, case.dt, case.steps, seed, case.notes)


def obstacle_course_1m(seed: int = 0) -> Case:
    """The 1M dam break with the 16k obstacle course scaled into its 4 x 2 x 2
    m box (positions by the box, sizes and field radii by 2): a tilted plane,
    a rotated box, a sphere, an upright cylinder, a lying capsule, a bounded
    wind, an unbounded vortex and a bounded point attractor. Falloffs are 1,
    where the reference's powf is exact."""
    case = dam_break_1m(seed)
    p = case.params
    add_collider(p, PLANE, pose((2.2, 0.1, 0.7), ((0.0, 0.0, 1.0), 0.35)))
    add_collider(p, BOX, pose((2.2, 0.24, 1.4), ((0.3, 1.0, 0.2), 0.6)), half_extents=(0.16, 0.2, 0.12))
    add_collider(p, SPHERE, pose((1.2, 0.2, 0.4)), radius=0.18)
    add_collider(p, CYLINDER, pose((3.2, 0.3, 1.0)), half_extents=(0.0, 0.3, 0.0), radius=0.14)
    add_collider(p, CAPSULE, pose((1.8, 0.16, 1.0), ((1.0, 0.0, 0.0), 1.5707964)), half_extents=(0.0, 0.24, 0.0),
                 radius=0.1)
    add_force_field(p, WIND, (2.0, 0.6, 1.0), (1.0, 0.0, 0.0), 3.0, radius=1.2, falloff=1.0)
    add_force_field(p, VORTEX, (2.0, 0.0, 1.0), (0.0, 1.0, 0.0), 4.0, radius=0.0)
    add_force_field(p, POINT, (2.8, 0.8, 1.0), (0.0, 0.0, 0.0), 5.0, radius=1.0, falloff=1.0)
    return Case("obstacle_course_1m", p, case.count, case.dt, case.steps, seed, case.notes)


def obstacles_small() -> SphParams:
    """2,048 particles (16 x 16 x 8) in a 0.6 m box with one collider of each
    shape and one field of each kind close to the block, so that every
    collider and field acts within a few substeps. Falloffs are 1, where the
    reference's powf is exact."""
    p = make_params(container_min=(0.0, 0.0, 0.0), container_max=(0.6, 0.6, 0.6), lattice=(16, 16, 8),
                    cell_count=4096)
    # The block spans about [0.02, 0.32] x [0.02, 0.32] x [0.02, 0.16].
    add_collider(p, SPHERE, pose((0.17, 0.17, 0.09)), radius=0.05)
    add_collider(p, BOX, pose((0.3, 0.05, 0.1), ((0.2, 1.0, 0.4), 0.7)), half_extents=(0.05, 0.04, 0.06))
    add_collider(p, PLANE, pose((0.3, 0.02, 0.3), ((1.0, 0.0, 1.0), 0.3)))
    add_collider(p, CYLINDER, pose((0.05, 0.1, 0.12)), half_extents=(0.0, 0.06, 0.0), radius=0.03)
    add_collider(p, CAPSULE, pose((0.25, 0.25, 0.05), ((0.0, 0.0, 1.0), 1.2)), half_extents=(0.0, 0.05, 0.0),
                 radius=0.025)
    add_collider(p, MESH, pose((0.5, 0.5, 0.5)))  # falls through to a point sphere, as in the reference
    add_force_field(p, WIND, (0.1, 0.2, 0.1), (0.0, 0.0, 1.0), 2.0, radius=0.3, falloff=1.0)
    add_force_field(p, VORTEX, (0.17, 0.0, 0.09), (0.0, 1.0, 0.0), 3.0, radius=0.0)
    add_force_field(p, POINT, (0.2, 0.3, 0.1), (0.0, 0.0, 0.0), 4.0, radius=0.25, falloff=1.0)
    return p


@dataclass
class TankSet:
    """Many independent tanks: per-tank constants, counts and initial states."""

    name: str
    params: list
    counts: list
    dt: float
    steps: int
    seed: int
    notes: str = ""

    def initial_state(self, tank: int):
        return jittered_block(self.params[tank], self.counts[tank], self.seed * 1_000_003 + tank)

    @property
    def total_particles(self) -> int:
        return int(sum(self.counts))


def _draws(seed: int, stream: int, count: int) -> np.ndarray:
    """`count` uniforms in [0, 1) from splitmix64, one stream per purpose."""
    return uniform01(seed * 7919 + stream, np.arange(count, dtype=np.uint64)).astype(np.float64)


def tank_lattice(n: int, extent, fill: float, spacing: float):
    """Block of `n` particles for one tank: nx = floor(f Lx / s),
    nz = floor(f Lz / s), ny = ceil(n / (nx nz)); while the block is taller
    than the tank allows (ny s > Ly - 2 s), nx and nz grow (within the walls)."""
    s = spacing
    nx = max(1, int(np.floor(fill * extent[0] / s)))
    nz = max(1, int(np.floor(fill * extent[2] / s)))
    max_x = max(1, int(np.floor((extent[0] - 2 * s) / s)))
    max_z = max(1, int(np.floor((extent[2] - 2 * s) / s)))
    ny = -(-n // (nx * nz))
    while ny * s > extent[1] - 2 * s and (nx < max_x or nz < max_z):
        if nx < max_x:
            nx += 1
        if nz < max_z:
            nz += 1
        ny = -(-n // (nx * nz))
    # The emit rule fills x, then y, then z (fluid_sph.cpp:147-149).
    layers = -(-n // (nx * ny))
    return nx, ny, layers


def batched_tanks(tanks: int = 256, seed: int = 0, spacing: float = 0.02) -> TankSet:
    """Independent dam-break tanks with uneven particle counts.

    Per tank: N log-uniform in [2048, 65536], extents uniform in [0.5, 2] m per
    axis, initial block fill fraction uniform in [0.2, 0.6], s = 0.02 m,
    h = 0.04 m, dt = 1/600 s, and the reference's bucket rule
    (gfx::cellCountFor). All draws are seeded splitmix64 streams.
    """
    u_n = _draws(seed, 1, tanks)
    u_l = _draws(seed, 2, 3 * tanks).reshape(tanks, 3)
    u_f = _draws(seed, 3, tanks)
    params, counts = [], []
    for t in range(tanks):
        n = int(round(np.exp(np.log(2048.0) + u_n[t] * (np.log(65536.0) - np.log(2048.0)))))
        extent = [float(np.float32(0.5 + 1.5 * u_l[t, a])) for a in range(3)]
        fill = 0.2 + 0.4 * u_f[t]
        lattice = tank_lattice(n, extent, fill, spacing)
        params.append(make_params(container_min=(0.0, 0.0, 0.0), container_max=extent, lattice=lattice,
                                  cell_count=cell_count_for(n), spacing=spacing))
        counts.append(n)
    return TankSet("batched_256_tanks", params, counts, 1.0 / 600.0, 300, seed,
                   "N_t log-uniform [2048, 65536], extents U[0.5, 2] m, fill U[0.2, 0.6]")
