// scene.h stand-in — declares only what the reference's fluid solver
// (src/physics/fluid_sph.{h,cpp}, force_field.h, collider_shapes.h) names
// from scene::, so those unmodified sources compile without the rest of the
// reference's scene module (which needs glm, assets and cameras).
// TEST INFRASTRUCTURE ONLY. Field names and enum values follow
// src/scene/scene.h (ColliderShape :119, Fluid :186-218, ForceFieldType
// :287, ForceField :295, ColliderPose :157).
#pragma once

#include <cstdint>
#include <vector>

#include <glm/mat4x4.hpp>
#include <glm/vec3.hpp>

namespace scene {

enum class SimulationBackend : uint32_t { AUTO = 0, CPU = 1, GPU = 2 };

enum class ColliderShape : uint32_t { SPHERE = 0, BOX = 1, PLANE = 2, CYLINDER = 3, CAPSULE = 4, MESH = 5 };

enum class ForceFieldType : uint32_t { WIND = 0, VORTEX = 1, POINT = 2 };

struct Fluid {
    glm::vec3 emitterHalfExtents{0.5F};
    uint32_t particleCount = 8192;
    float particleRadius = 0.025F;
    float smoothingRadius = 0.1F;
    float restDensity = 1000.0F;
    float stiffness = 50.0F;
    float viscosity = 0.5F;
    glm::vec3 containerMin{-1.0F, 0.0F, -1.0F};
    glm::vec3 containerMax{1.0F, 2.0F, 1.0F};
    glm::vec3 gravity{0.0F, -9.81F, 0.0F};
};

struct RigidBody {
    ColliderShape shape = ColliderShape::SPHERE;
    float radius = 0.5F;
    glm::vec3 halfExtents{0.5F};
};

struct ForceField {
    ForceFieldType type = ForceFieldType::WIND;
    float strength = 5.0F;
    float radius = 0.0F;
    float falloff = 1.0F;
};

struct ColliderPose {
    glm::vec3 position{0.0F};
    glm::quat rotation{1.0F, 0.0F, 0.0F, 0.0F};
    float radius = 0.0F;
    glm::vec3 halfExtents{0.0F};
    glm::vec3 scale{1.0F};
};

ColliderPose colliderPose(const RigidBody& body, const glm::mat4& world);

struct Object {
    int32_t rigidBody = -1;
    int32_t forceField = -1;
};

// An empty scene: the checker derives parameters with no colliders and no
// force fields.
struct Scene {
    std::vector<Object> objects;
    std::vector<RigidBody> rigidBodies;
    std::vector<ForceField> forceFields;
    std::vector<glm::mat4> cachedWorlds;
    std::vector<uint8_t> cachedVisible;
    const glm::mat4& world(uint32_t index) const { return cachedWorlds[index]; }
    bool visibleCached(uint32_t index) const { return cachedVisible[index] != 0; }
};

} // namespace scene
