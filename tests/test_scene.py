"""Scene files for fluids (computer_graphics_lab_00_gb300/scene.py): reading
and writing the version-2 document, the solver constants derived from a
scene against physics::deriveFluidParams, object transforms, colliders and
force fields collected from scene objects; on the GPU, a scene run headless
against the oracle stepping the same constants."""
from __future__ import annotations

import json
import math
import numpy as np
import pytest

from computer_graphics_lab_00_gb300 import scene as S
from computer_graphics_lab_00_gb300 import workloads as W
from oracle.bind import REFERENCE_TREE

REFERENCE_SCENES = REFERENCE_TREE / "tests" / "scenes"


def demo_scene(display="particles", count=4096) -> S.Scene:
    sc = S.Scene(name="demo")
    sc.fluids.append(S.FluidSettings(particle_count=count, display=display, emitter_half_extents=(0.3, 0.3, 0.3),
                                     surface_resolution=40))
    sc.rigid_bodies += [S.RigidBody(shape="plane", kinematic=True),
                        S.RigidBody(shape="sphere", radius=0.25),
                        S.RigidBody(shape="box", half_extents=(0.2, 0.1, 0.3)),
                        S.RigidBody(shape="capsule", radius=0.1, half_extents=(0.0, 0.2, 0.0)),
                        S.RigidBody(shape="mesh")]
    sc.force_fields.append(S.ForceField(type="vortex", strength=2.0, radius=0.0))
    half = math.sqrt(0.5)
    sc.objects += [
        S.SceneObject(name="water", position=(0.0, 1.0, 0.0), fluid=0),
        S.SceneObject(name="floor", position=(0.0, 0.05, 0.0), rotation=(0.0, 0.0, 0.05, math.sqrt(1 - 0.0025)),
                      rigid_body=0),
        S.SceneObject(name="ball", position=(0.3, 0.3, 0.2), rigid_body=1),
        S.SceneObject(name="crate", position=(-0.4, 0.2, -0.3), rotation=(0.0, half, 0.0, half),
                      scale=(1.5, 1.0, 1.0), rigid_body=2),
        S.SceneObject(name="arm", parent=3, position=(0.0, 0.4, 0.0), rotation=(half, 0.0, 0.0, half),
                      rigid_body=3),
        S.SceneObject(name="statue", position=(0.5, 0.5, 0.5), rigid_body=4),
        S.SceneObject(name="hidden ball", position=(0.0, 0.5, 0.0), visible=False, rigid_body=1),
        S.SceneObject(name="swirl", position=(0.0, 0.0, 0.0), force_field=0),
    ]
    return sc


def test_document_round_trip(tmp_path):
    sc = demo_scene()
    path = tmp_path / "scene.json"
    S.save_scene(sc, path)
    again = S.load_scene(path)
    assert S.scene_document(again) == S.scene_document(sc)
    doc = json.loads(path.read_text())
    doc["objects"].append({"name": "dangling", "fluid": 7, "rigidBody": -3})  # out-of-range parts drop
    doc["fluids"][0]["surfaceResolution"] = 1000  # clamped to [8, 128] like scene_io.cpp:580
    loaded = S.load_scene(doc)
    assert loaded.objects[-1].fluid == -1 and loaded.objects[-1].rigid_body == -1
    assert loaded.fluids[0].surface_resolution == 128


def settings_struct(settings):
    s = S.abi.SphFluidSettings()
    s.emitter_half_extents[:] = settings.emitter_half_extents
    s.particle_radius = settings.particle_radius
    s.smoothing_radius = settings.smoothing_radius
    s.rest_density = settings.rest_density
    s.stiffness = settings.stiffness
    s.viscosity = settings.viscosity
    s.container_min[:] = settings.container_min
    s.container_max[:] = settings.container_max
    s.gravity[:] = settings.gravity
    return s


def test_constants_match_derive_fluid_params(native, oracle):
    """The reference test scene (emitter at (0, 1, 0)) gives exactly the
    constants of the oracle's deriveFluidParams, and the workload generator's
    physics (it differs only in the emitter half extents, which emit does not
    read: the generator derives them from the lattice)."""
    sc = S.Scene()
    sc.fluids.append(S.FluidSettings(particle_count=1024))
    sc.objects.append(S.SceneObject(position=(0.0, 1.0, 0.0), fluid=0))
    params, count, owner = S.fluid_params(sc, 0, cell_count=1024)
    assert count == 1024 and owner == 0
    want = oracle.derive_params(settings_struct(sc.fluids[0]), S.column_major(sc.world(0)), 1024, 1024)
    assert bytes(params) == bytes(want)
    generated = W.reference_test_scene(1024)
    generated.emitter_half_extents[:3] = params.emitter_half_extents[:3]
    assert bytes(params) == bytes(generated)


def test_particle_limit_and_unowned_fluid(native):
    sc = S.Scene()
    sc.fluids += [S.FluidSettings(particle_count=100000), S.FluidSettings()]
    sc.objects.append(S.SceneObject(fluid=0))
    params, count, _ = S.fluid_params(sc, 0)
    assert count == S.FLUID_MAX_PARTICLES and params.lattice[3] == 65536
    assert S.fluid_params(sc, 1) == (None, 0, -1)


def test_transforms_follow_glm():
    # mat3_cast of a unit quaternion is a rotation; composition with parents.
    q = np.array([0.1, -0.3, 0.2, 0.9])
    q = q / np.linalg.norm(q)
    r = S.quat_to_matrix(q).astype(np.float64)
    np.testing.assert_allclose(r.T @ r, np.eye(3), atol=1e-6)
    x, y, z, w = q
    expected = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
                         [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
                         [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]])
    np.testing.assert_allclose(r, expected, atol=1e-6)
    sc = demo_scene()
    arm = sc.world(4).astype(np.float64)
    parent = S.transform_matrix(*(getattr(sc.objects[3], k) for k in ("position", "rotation", "scale")))
    local = S.transform_matrix(*(getattr(sc.objects[4], k) for k in ("position", "rotation", "scale")))
    np.testing.assert_allclose(arm, parent.astype(np.float64) @ local.astype(np.float64), atol=1e-6)
    assert sc.visible(0) and not sc.visible(6)


def test_colliders_and_fields_from_objects(native):
    sc = demo_scene()
    params, _, _ = S.fluid_params(sc, 0)
    # floor, ball, crate, arm; the mesh statue and the hidden ball are left out.
    assert params.collider_count == 4
    assert [params.colliders[k].type for k in range(4)] == [2, 0, 1, 4]
    ball = params.colliders[1]
    assert ball.data0[3] == pytest.approx(0.25)
    np.testing.assert_allclose([ball.world[12], ball.world[13], ball.world[14]], (0.3, 0.3, 0.2), atol=1e-7)
    crate = params.colliders[2]
    np.testing.assert_allclose(crate.data0[:3], (0.3, 0.1, 0.3), atol=1e-6)  # half extents times scale
    world = np.array(crate.world, np.float64).reshape(4, 4).T
    inverse = np.array(crate.inverse_world, np.float64).reshape(4, 4).T
    np.testing.assert_allclose(world @ inverse, np.eye(4), atol=1e-6)
    arm = params.colliders[3]
    np.testing.assert_allclose([arm.world[12], arm.world[13], arm.world[14]], (-0.4, 0.6, -0.3), atol=1e-6)
    assert params.field_count == 1
    f = params.fields[0]
    assert f.type == 1 and f.position_radius[3] == 0.0
    np.testing.assert_allclose(f.axis_strength[:3], (0.0, 1.0, 0.0), atol=1e-7)


@pytest.mark.parametrize("name", ["fluid.json", "fluid_surface.json", "fluid_surface_cpu.json"])
def test_reference_scene_files_load(native, reference_available, name):
    """The reference's own fluid scenes read and give the constants its
    deriveFluidParams gives for the same settings and emitter matrix."""
    if not reference_available or not (REFERENCE_SCENES / name).exists():
        pytest.skip("reference tree absent")
    from oracle.bind import Reference

    sc = S.load_scene(REFERENCE_SCENES / name)
    assert sc.fluids
    params, count, owner = S.fluid_params(sc, 0)
    assert count > 0
    ref = Reference().derive_params(settings_struct(sc.fluids[0]), S.column_major(sc.world(owner)), count,
                                    params.lattice[3])
    head = S.abi.SphParams.collider_count.offset
    assert bytes(params)[:head] == bytes(ref)[:head]


@pytest.mark.gpu
@pytest.mark.parametrize("display", ["particles", "surface"])
def test_scene_runs_headless_like_the_oracle(native, oracle, tmp_path, display):
    sc = demo_scene(display=display, count=4096)
    path = tmp_path / "scene.json"
    S.save_scene(sc, path)
    results = S.run_scene(path, frames=20, out_dir=tmp_path)
    params, count, _ = S.fluid_params(sc, 0)
    pos, vel = oracle.emit(params, count)
    pos, vel = oracle.step(params, pos, vel, 1.0 / 60.0, threads=oracle.hardware_threads, frames=20)
    got = np.load(tmp_path / "fluid0_particles.npy")
    np.testing.assert_array_equal(got.view(np.uint32), pos.view(np.uint32))
    assert results[0]["colliders"] == 4 and results[0]["force_fields"] == 1
    if display == "surface":
        assert results[0]["surface_vertices"] > 0
        text = (tmp_path / "fluid0_surface.obj").read_text()
        assert text.count("\nf ") * 3 == results[0]["surface_vertices"]
