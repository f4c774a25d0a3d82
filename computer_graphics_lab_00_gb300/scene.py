"""Scene files for fluids: read, write, derive solver constants, run headless.

Reads the fluid-relevant part of the reference's scene JSON (version 2,
src/scene/scene_io.cpp): `fluids` (:562-586), `rigidBodies` (:548-560),
`forceFields` (:607-617) and `objects` (:698-712, with the same handling of
indices that point outside their arrays). `fluid_params` turns one fluid into
the solver's constants as the reference's renderer does per frame
(FluidSimulator::deriveParams, src/gfx/fluid.cpp:335-369 and :507-509 ->
physics::deriveFluidParams, fluid_sph.cpp:65-126): particle count capped at
FLUID_MAX_PARTICLES, bucket count from the particle count, emitter placed by
the owning object's world matrix, shape colliders from visible rigid bodies
(collectShapeColliders) and force fields from visible force-field objects
(collectForceFields, force_field.h:73-93). `run_scene` steps every fluid of a
scene headlessly on the GPU at a fixed frame time and writes particles and,
for surface fluids, the marching-cubes mesh to files: there is no window.

Exactness: the fluid constants come from sph_derive_params and match the
reference bit for bit; an object's world matrix follows Transform::matrix
(scene.cpp:74-78) in float32 with glm's quaternion-to-matrix formula.
Collider poses need glm::decompose and glm::inverse, which are evaluated here
in float64 and rounded to float32 (glm is not available to pin them).
"""
from __future__ import annotations

import json
import math
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from . import abi

SHAPES = ("sphere", "box", "plane", "cylinder", "capsule", "mesh")
FIELD_TYPES = ("wind", "vortex", "point")
BACKENDS = ("auto", "cpu", "gpu")
FLUID_MAX_PARTICLES = 32768        # src/gfx/fluid.h:27
SURFACE_RESOLUTION_RANGE = (8, 128)  # scene_io.cpp:580
F32 = np.float32


@dataclass
class FluidSettings:
    """scene::Fluid (src/scene/scene.h:186-218) with its defaults."""

    backend: str = "auto"
    display: str = "particles"
    emitter_half_extents: tuple = (0.5, 0.5, 0.5)
    particle_count: int = 8192
    particle_radius: float = 0.025
    smoothing_radius: float = 0.1
    rest_density: float = 1000.0
    stiffness: float = 50.0
    viscosity: float = 0.5
    container_min: tuple = (-1.0, 0.0, -1.0)
    container_max: tuple = (1.0, 2.0, 1.0)
    gravity: tuple = (0.0, -9.81, 0.0)
    surface_resolution: int = 48
    surface_iso: float = 0.5
    surface_roughness: float = 0.05
    water_color: tuple = (0.35, 0.65, 0.75)
    absorption: tuple = (2.2, 0.5, 0.25)
    thickness_scale: float = 1.0


@dataclass
class RigidBody:
    """The parts of scene::RigidBody (scene.h:130-150) a fluid sees."""

    shape: str = "sphere"
    backend: str = "auto"
    mass: float = 1.0
    use_gravity: bool = True
    kinematic: bool = False
    restitution: float = 0.3
    friction: float = 0.5
    radius: float = 0.5
    half_extents: tuple = (0.5, 0.5, 0.5)


@dataclass
class ForceField:
    """scene::ForceField (scene.h:295-305)."""

    type: str = "wind"
    strength: float = 5.0
    radius: float = 0.0
    falloff: float = 1.0


@dataclass
class SceneObject:
    name: str = "object"
    parent: int = -1
    position: tuple = (0.0, 0.0, 0.0)
    rotation: tuple = (0.0, 0.0, 0.0, 1.0)  # x, y, z, w as in the file
    scale: tuple = (1.0, 1.0, 1.0)
    visible: bool = True
    rigid_body: int = -1
    fluid: int = -1
    force_field: int = -1


@dataclass
class Scene:
    name: str = ""
    fluids: list = field(default_factory=list)
    rigid_bodies: list = field(default_factory=list)
    force_fields: list = field(default_factory=list)
    objects: list = field(default_factory=list)

    # -- transforms (scene.cpp:74-78, :413-429) --------------------------------------------
    def local_matrix(self, index: int) -> np.ndarray:
        o = self.objects[index]
        return transform_matrix(o.position, o.rotation, o.scale)

    def world(self, index: int) -> np.ndarray:
        """Column-major float32 4x4 (as a numpy [4, 4] with m[:, c] column c)."""
        world = self.local_matrix(index)
        parent = self.objects[index].parent
        guard = 0
        while 0 <= parent < len(self.objects) and guard <= len(self.objects):
            world = matmul_f32(self.local_matrix(parent), world)
            parent = self.objects[parent].parent
            guard += 1
        return world

    def visible(self, index: int) -> bool:
        current = index
        guard = 0
        while 0 <= current < len(self.objects) and guard <= len(self.objects):
            if not self.objects[current].visible:
                return False
            current = self.objects[current].parent
            guard += 1
        return True


# ---- float32 matrix helpers in glm's evaluation order ------------------------------------

def quat_to_matrix(q) -> np.ndarray:
    """glm::mat3_cast of a quaternion (x, y, z, w), float32, as [3, 3] with
    m[:, c] column c."""
    x, y, z, w = (F32(v) for v in q)
    qxx, qyy, qzz = x * x, y * y, z * z
    qxz, qxy, qyz = x * z, x * y, y * z
    qwx, qwy, qwz = w * x, w * y, w * z
    one, two = F32(1.0), F32(2.0)
    m = np.empty((3, 3), np.float32)
    m[0, 0] = one - two * (qyy + qzz)
    m[1, 0] = two * (qxy + qwz)
    m[2, 0] = two * (qxz - qwy)
    m[0, 1] = two * (qxy - qwz)
    m[1, 1] = one - two * (qxx + qzz)
    m[2, 1] = two * (qyz + qwx)
    m[0, 2] = two * (qxz + qwy)
    m[1, 2] = two * (qyz - qwx)
    m[2, 2] = one - two * (qxx + qyy)
    return m


def transform_matrix(position, rotation, scale) -> np.ndarray:
    """Transform::matrix: translate(I, p) * mat4_cast(q), then scale's columns."""
    m = np.zeros((4, 4), np.float32)
    r = quat_to_matrix(rotation)
    for c in range(3):
        m[:3, c] = r[:, c] * F32(scale[c])
    m[:3, 3] = np.asarray(position, np.float32)
    m[3, 3] = F32(1.0)
    return m


def matmul_f32(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """glm mat4 * mat4: each result column is a * column, (c0 x + c1 y) + (c2 z + c3 w)."""
    out = np.empty((4, 4), np.float32)
    for c in range(4):
        v = b[:, c]
        out[:, c] = (a[:, 0] * v[0] + a[:, 1] * v[1]) + (a[:, 2] * v[2] + a[:, 3] * v[3])
    return out


def column_major(m: np.ndarray) -> list:
    return [float(m[r, c]) for c in range(4) for r in range(4)]


# ---- reading and writing ------------------------------------------------------------------

def _vec(value, default, n=3):
    if isinstance(value, list) and len(value) == n:
        return tuple(float(v) for v in value)
    return tuple(default)


def _quat(value):
    if isinstance(value, list) and len(value) == 4:
        return tuple(float(v) for v in value)
    return (0.0, 0.0, 0.0, 1.0)


def _index(value, size):
    return value if isinstance(value, int) and 0 <= value < size else -1


def load_scene(source) -> Scene:
    """A Scene from a path or an already parsed JSON document."""
    doc = source if isinstance(source, dict) else json.loads(Path(source).read_text(encoding="utf-8"))
    scene = Scene(name=doc.get("name", ""))
    for e in doc.get("rigidBodies", []):
        d = RigidBody()
        scene.rigid_bodies.append(RigidBody(
            shape=e.get("shape", "sphere") if e.get("shape", "sphere") in SHAPES else "sphere",
            backend=e.get("backend", "auto") if e.get("backend", "auto") in BACKENDS else "auto",
            mass=float(e.get("mass", d.mass)), use_gravity=bool(e.get("useGravity", d.use_gravity)),
            kinematic=bool(e.get("kinematic", d.kinematic)), restitution=float(e.get("restitution", d.restitution)),
            friction=float(e.get("friction", d.friction)), radius=float(e.get("radius", d.radius)),
            half_extents=_vec(e.get("halfExtents"), d.half_extents)))
    for e in doc.get("fluids", []):
        d = FluidSettings()
        lo, hi = SURFACE_RESOLUTION_RANGE
        scene.fluids.append(FluidSettings(
            backend=e.get("backend", "auto") if e.get("backend", "auto") in BACKENDS else "auto",
            display="surface" if e.get("display", "particles") == "surface" else "particles",
            emitter_half_extents=_vec(e.get("emitterHalfExtents"), d.emitter_half_extents),
            particle_count=int(e.get("particleCount", d.particle_count)),
            particle_radius=float(e.get("particleRadius", d.particle_radius)),
            smoothing_radius=float(e.get("smoothingRadius", d.smoothing_radius)),
            rest_density=float(e.get("restDensity", d.rest_density)),
            stiffness=float(e.get("stiffness", d.stiffness)), viscosity=float(e.get("viscosity", d.viscosity)),
            container_min=_vec(e.get("containerMin"), d.container_min),
            container_max=_vec(e.get("containerMax"), d.container_max),
            gravity=_vec(e.get("gravity"), d.gravity),
            surface_resolution=min(max(int(e.get("surfaceResolution", d.surface_resolution)), lo), hi),
            surface_iso=float(e.get("surfaceIso", d.surface_iso)),
            surface_roughness=float(e.get("surfaceRoughness", d.surface_roughness)),
            water_color=_vec(e.get("waterColor"), d.water_color), absorption=_vec(e.get("absorption"), d.absorption),
            thickness_scale=float(e.get("thicknessScale", d.thickness_scale))))
    for e in doc.get("forceFields", []):
        t = e.get("type", "wind")
        scene.force_fields.append(ForceField(
            type=t if t in FIELD_TYPES else "wind", strength=float(e.get("strength", 5.0)),
            radius=max(float(e.get("radius", 0.0)), 0.0), falloff=max(float(e.get("falloff", 1.0)), 0.0)))
    for e in doc.get("objects", []):
        scene.objects.append(SceneObject(
            name=e.get("name", "object"), parent=int(e.get("parent", -1)),
            position=_vec(e.get("position"), (0.0, 0.0, 0.0)), rotation=_quat(e.get("rotation")),
            scale=_vec(e.get("scale"), (1.0, 1.0, 1.0)), visible=bool(e.get("visible", True)),
            rigid_body=_index(e.get("rigidBody", -1), len(scene.rigid_bodies)),
            fluid=_index(e.get("fluid", -1), len(scene.fluids)),
            force_field=_index(e.get("forceField", -1), len(scene.force_fields))))
    return scene


def scene_document(scene: Scene) -> dict:
    """The fluid-relevant part of a version-2 scene document (scene_io.cpp:200-282)."""
    return {
        "version": 2,
        "name": scene.name,
        "rigidBodies": [{"backend": b.backend, "shape": b.shape, "mass": b.mass, "useGravity": b.use_gravity,
                         "kinematic": b.kinematic, "restitution": b.restitution, "friction": b.friction,
                         "radius": b.radius, "halfExtents": list(b.half_extents)} for b in scene.rigid_bodies],
        "fluids": [{"backend": f.backend, "emitterHalfExtents": list(f.emitter_half_extents),
                    "particleCount": f.particle_count, "particleRadius": f.particle_radius,
                    "smoothingRadius": f.smoothing_radius, "restDensity": f.rest_density, "stiffness": f.stiffness,
                    "viscosity": f.viscosity, "containerMin": list(f.container_min),
                    "containerMax": list(f.container_max), "gravity": list(f.gravity), "display": f.display,
                    "surfaceResolution": f.surface_resolution, "surfaceIso": f.surface_iso,
                    "surfaceRoughness": f.surface_roughness, "waterColor": list(f.water_color),
                    "absorption": list(f.absorption), "thicknessScale": f.thickness_scale} for f in scene.fluids],
        "forceFields": [{"type": f.type, "strength": f.strength, "radius": f.radius, "falloff": f.falloff}
                        for f in scene.force_fields],
        "objects": [dict({"name": o.name, "parent": o.parent, "position": list(o.position),
                          "rotation": list(o.rotation), "scale": list(o.scale), "visible": o.visible},
                         **({"rigidBody": o.rigid_body} if o.rigid_body >= 0 else {}),
                         **({"fluid": o.fluid} if o.fluid >= 0 else {}),
                         **({"forceField": o.force_field} if o.force_field >= 0 else {}))
                    for o in scene.objects],
    }


def save_scene(scene: Scene, path) -> None:
    Path(path).write_text(json.dumps(scene_document(scene), indent=2, ensure_ascii=False), encoding="utf-8")


# ---- solver constants ----------------------------------------------------------------------

def _collider_pose(body: RigidBody, world: np.ndarray):
    """scene::colliderPose (scene.cpp:254-268): position, unit rotation and
    scaled extents from the world matrix (decomposed in float64)."""
    m = world.astype(np.float64)
    position = m[:3, 3]
    basis = m[:3, :3].copy()
    scale = np.linalg.norm(basis, axis=0)
    if np.linalg.det(basis) < 0:
        scale = -scale
    rot = basis / np.where(scale == 0, 1.0, scale)
    # Rotation matrix -> quaternion (Shepperd's method), then normalised.
    t = np.trace(rot)
    if t > 0:
        s = math.sqrt(t + 1.0) * 2
        q = ((rot[2, 1] - rot[1, 2]) / s, (rot[0, 2] - rot[2, 0]) / s, (rot[1, 0] - rot[0, 1]) / s, 0.25 * s)
    elif rot[0, 0] > rot[1, 1] and rot[0, 0] > rot[2, 2]:
        s = math.sqrt(1.0 + rot[0, 0] - rot[1, 1] - rot[2, 2]) * 2
        q = (0.25 * s, (rot[0, 1] + rot[1, 0]) / s, (rot[0, 2] + rot[2, 0]) / s, (rot[2, 1] - rot[1, 2]) / s)
    elif rot[1, 1] > rot[2, 2]:
        s = math.sqrt(1.0 + rot[1, 1] - rot[0, 0] - rot[2, 2]) * 2
        q = ((rot[0, 1] + rot[1, 0]) / s, 0.25 * s, (rot[1, 2] + rot[2, 1]) / s, (rot[0, 2] - rot[2, 0]) / s)
    else:
        s = math.sqrt(1.0 + rot[2, 2] - rot[0, 0] - rot[1, 1]) * 2
        q = ((rot[0, 2] + rot[2, 0]) / s, (rot[1, 2] + rot[2, 1]) / s, 0.25 * s, (rot[1, 0] - rot[0, 1]) / s)
    q = np.asarray(q) / np.linalg.norm(q)
    radius = body.radius * (max(scale[0], scale[2]) if body.shape in ("cylinder", "capsule") else max(scale))
    half = np.asarray(body.half_extents) * scale
    return position, q, float(radius), half


def fluid_params(scene: Scene, fluid_index: int, particle_limit: int = FLUID_MAX_PARTICLES,
                 cell_count: int | None = None):
    """(SphParams, particle count, owning object index) of one fluid, as the
    reference's renderer derives them; count 0 when no object owns the fluid."""
    from .fluid import derive_fluid_params
    from .workloads import cell_count_for

    owners = [i for i, o in enumerate(scene.objects) if o.fluid == fluid_index]
    settings = scene.fluids[fluid_index]
    if not owners:
        return None, 0, -1
    owner = owners[0]
    count = min(settings.particle_count, particle_limit)
    world = scene.world(owner) if scene.visible(owner) else np.zeros((4, 4), np.float32)
    s = abi.SphFluidSettings()
    s.emitter_half_extents[:] = settings.emitter_half_extents
    s.particle_radius = settings.particle_radius
    s.smoothing_radius = settings.smoothing_radius
    s.rest_density = settings.rest_density
    s.stiffness = settings.stiffness
    s.viscosity = settings.viscosity
    s.container_min[:] = settings.container_min
    s.container_max[:] = settings.container_max
    s.gravity[:] = settings.gravity
    params = derive_fluid_params(s, column_major(world), count, cell_count or cell_count_for(count))
    # collectShapeColliders (fluid_sph.cpp:102-126).
    k = 0
    for i, o in enumerate(scene.objects):
        if k >= abi.SPH_MAX_COLLIDERS:
            break
        if o.rigid_body < 0 or not scene.visible(i):
            continue
        body = scene.rigid_bodies[o.rigid_body]
        if body.shape == "mesh":
            continue
        position, q, radius, half = _collider_pose(body, scene.world(i))
        rigid = np.eye(4)
        rigid[:3, :3] = quat_to_matrix(q).astype(np.float64)
        rigid[:3, 3] = position
        c = params.colliders[k]
        rigid32 = rigid.astype(np.float32)
        inverse32 = np.linalg.inv(rigid).astype(np.float32)
        for col in range(4):
            for r in range(4):
                c.world[col * 4 + r] = float(rigid32[r, col])
                c.inverse_world[col * 4 + r] = float(inverse32[r, col])
        c.data0[0], c.data0[1], c.data0[2] = (float(F32(v)) for v in half)
        c.data0[3] = float(F32(radius))
        c.type = SHAPES.index(body.shape)
        k += 1
    params.collider_count = k
    # collectForceFields (force_field.h:73-93).
    k = 0
    for i, o in enumerate(scene.objects):
        if k >= abi.SPH_MAX_FORCE_FIELDS:
            break
        if o.force_field < 0 or not scene.visible(i):
            continue
        ff = scene.force_fields[o.force_field]
        w = scene.world(i)
        axis = w[:3, 1].copy() if ff.type == "vortex" else -w[:3, 2]
        length = np.sqrt((axis[0] * axis[0] + axis[1] * axis[1]) + axis[2] * axis[2])
        axis = axis / length if length > F32(1e-6) else np.array([0.0, 1.0, 0.0], np.float32)
        f = params.fields[k]
        f.position_radius[:3] = [float(v) for v in w[:3, 3]]
        f.position_radius[3] = max(ff.radius, 0.0)
        f.axis_strength[:3] = [float(v) for v in axis]
        f.axis_strength[3] = ff.strength
        f.falloff = max(ff.falloff, 0.0)
        f.type = FIELD_TYPES.index(ff.type)
        k += 1
    params.field_count = k
    return params, count, owner


# ---- headless run --------------------------------------------------------------------------

def unpack_unit_vector(packed) -> np.ndarray:
    """asset::unpackUnitVector (vertex_pack.h:53-60) for an array of packed normals."""
    packed = np.asarray(packed, np.uint32)
    fx = np.clip((packed & 0xFFFF).astype(np.int16).astype(np.float32) / F32(32767.0), -1, 1)
    fy = np.clip(((packed >> 16) & 0xFFFF).astype(np.int16).astype(np.float32) / F32(32767.0), -1, 1)
    n = np.stack([fx, fy, F32(1.0) - np.abs(fx) - np.abs(fy)], axis=1)
    t = np.clip(-n[:, 2], 0, 1)
    n[:, 0] += np.where(n[:, 0] >= 0, -t, t)
    n[:, 1] += np.where(n[:, 1] >= 0, -t, t)
    return n / np.linalg.norm(n, axis=1, keepdims=True)


def write_obj(path, vertices) -> None:
    """Triangle soup as Wavefront OBJ with per-vertex normals."""
    p = vertices["position"]
    n = unpack_unit_vector(vertices["normal"])
    lines = [f"v {a:.7g} {b:.7g} {c:.7g}" for a, b, c in p]
    lines += [f"vn {a:.7g} {b:.7g} {c:.7g}" for a, b, c in n]
    lines += [f"f {i + 1}//{i + 1} {i + 2}//{i + 2} {i + 3}//{i + 3}" for i in range(0, len(p) - len(p) % 3, 3)]
    Path(path).write_text("\n".join(lines) + "\n")


def run_scene(source, frames: int = 120, frame_dt: float = 1.0 / 60.0, out_dir=None, device: int = 0,
              particle_limit: int = FLUID_MAX_PARTICLES, surface_capacity: int = 196608) -> list:
    """Emits and steps every fluid of a scene for `frames` frames on the GPU
    (FluidSolver::emit / step through the C ABI). With out_dir, writes
    fluid<i>_particles.npy and, for surface fluids, fluid<i>_surface.obj."""
    from .fluid import FluidSolverGpu

    scene = load_scene(source)
    results = []
    for index in range(len(scene.fluids)):
        params, count, owner = fluid_params(scene, index, particle_limit)
        if count == 0:
            results.append({"fluid": index, "particles": 0})
            continue
        settings = scene.fluids[index]
        with FluidSolverGpu(params, count, device=device) as solver:
            solver.emit(params, count)
            for _ in range(frames):
                solver.step(params, frame_dt)
            pos = solver.particles()
            entry = {"fluid": index, "object": owner, "particles": count, "colliders": params.collider_count,
                     "force_fields": params.field_count, "frames": frames}
            vertices = None
            if settings.display == "surface":
                vertices = solver.surface(settings.surface_resolution, settings.surface_iso, surface_capacity)
                entry["surface_vertices"] = int(len(vertices))
        if out_dir is not None:
            out = Path(out_dir)
            out.mkdir(parents=True, exist_ok=True)
            np.save(out / f"fluid{index}_particles.npy", pos)
            if vertices is not None:
                write_obj(out / f"fluid{index}_surface.obj", vertices)
        entry["mean_height"] = float(pos[:, 1].mean())
        results.append(entry)
    return results


def main() -> None:
    """python -m computer_graphics_lab_00_gb300.scene SCENE.json [--frames N] [--out DIR]"""
    import argparse

    ap = argparse.ArgumentParser(description=main.__doc__)
    ap.add_argument("scene")
    ap.add_argument("--frames", type=int, default=120)
    ap.add_argument("--frame-dt", type=float, default=1.0 / 60.0)
    ap.add_argument("--out", default=None)
    ap.add_argument("--particle-limit", type=int, default=FLUID_MAX_PARTICLES)
    args = ap.parse_args()
    print(json.dumps(run_scene(args.scene, args.frames, args.frame_dt, args.out, particle_limit=args.particle_limit),
                     indent=1))


if __name__ == "__main__":
    main()
