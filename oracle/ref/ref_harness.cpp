// ref_harness.cpp — C entry points over the reference's own, unmodified
// physics::FluidSolver / FluidGrid / deriveFluidParams / fluidSubsteps
// (src/physics/fluid_sph.{h,cpp}), compiled in place from the reference tree
// with the glm and scene stand-ins under oracle/ref/shim.
//
// TEST INFRASTRUCTURE ONLY: it pins the restated oracle (oracle/sph_oracle.cpp)
// against the reference. Harness hack: FluidSolver keeps its particle vectors
// private and offers no way to load a jittered state, so this translation
// unit alone reads the class with `private` spelled `public`. Only access
// changes; all data members sit in one access section, so the layout is the
// one the reference's own translation unit uses.
#include <algorithm>
#include <array>
#include <atomic>
#include <condition_variable>
#include <cstdint>
#include <cstring>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#define private public
#include "physics/fluid_sph.h"
#undef private

#include "core/job_system.h"
#include "physics/marching_cubes.h"
#include "sph_c.h"

namespace scene {
// Never reached: the checker's scenes hold no rigid bodies.
ColliderPose colliderPose(const RigidBody& body, const glm::mat4& world) {
    (void)body;
    (void)world;
    return ColliderPose{};
}
} // namespace scene

namespace {

physics::FluidParams toReference(const sph_params& p) {
    physics::FluidParams out;
    for (int c = 0; c < 4; ++c) {
        for (int r = 0; r < 4; ++r) {
            out.emitterWorld[c][r] = p.emitter_world[c * 4 + r];
        }
    }
    out.emitterHalfExtents = glm::vec3{p.emitter_half_extents[0], p.emitter_half_extents[1], p.emitter_half_extents[2]};
    out.spacing = p.emitter_half_extents[3];
    out.containerMin = glm::vec3{p.container_min[0], p.container_min[1], p.container_min[2]};
    out.particleRadius = p.container_min[3];
    out.containerMax = glm::vec3{p.container_max[0], p.container_max[1], p.container_max[2]};
    out.wallRestitution = p.container_max[3];
    out.gravity = glm::vec3{p.gravity[0], p.gravity[1], p.gravity[2]};
    out.particleMass = p.gravity[3];
    out.smoothingRadius = p.smoothing_radius;
    out.restDensity = p.rest_density;
    out.stiffness = p.stiffness;
    out.viscosity = p.viscosity;
    out.lattice = glm::uvec3{p.lattice[0], p.lattice[1], p.lattice[2]};
    out.cellCount = p.lattice[3];
    out.colliderCount = std::min<uint32_t>(p.collider_count, physics::FLUID_MAX_COLLIDERS);
    for (uint32_t c = 0; c < out.colliderCount; ++c) {
        const sph_collider& src = p.colliders[c];
        physics::FluidCollider& dst = out.colliders[c];
        dst.shape = static_cast<scene::ColliderShape>(src.type);
        dst.radius = src.data0[3];
        dst.halfExtents = glm::vec3{src.data0[0], src.data0[1], src.data0[2]};
        for (int col = 0; col < 4; ++col) {
            for (int r = 0; r < 4; ++r) {
                dst.world[col][r] = src.world[col * 4 + r];
                dst.inverseWorld[col][r] = src.inverse_world[col * 4 + r];
            }
        }
    }
    out.fieldCount = std::min<uint32_t>(p.field_count, physics::MAX_FORCE_FIELDS);
    for (uint32_t f = 0; f < out.fieldCount; ++f) {
        const sph_force_field& src = p.fields[f];
        physics::ForceFieldSample& dst = out.fields[f];
        dst.position = glm::vec3{src.position_radius[0], src.position_radius[1], src.position_radius[2]};
        dst.radius = src.position_radius[3];
        dst.axis = glm::vec3{src.axis_strength[0], src.axis_strength[1], src.axis_strength[2]};
        dst.strength = src.axis_strength[3];
        dst.falloff = src.falloff;
        dst.type = static_cast<scene::ForceFieldType>(src.type);
    }
    return out;
}

// One JobSystem per worker count, kept for the life of the library.
core::JobSystem* jobsFor(uint32_t threads) {
    static std::mutex guard;
    static std::map<uint32_t, std::unique_ptr<core::JobSystem>> systems;
    if (threads <= 1) {
        return nullptr;
    }
    std::lock_guard<std::mutex> lock(guard);
    std::unique_ptr<core::JobSystem>& slot = systems[threads];
    if (!slot) {
        slot = std::make_unique<core::JobSystem>(threads - 1);
    }
    return slot.get();
}

void copyIn(std::vector<glm::vec4>& dst, const float* src, uint32_t count) {
    dst.assign(count, glm::vec4{0.0F});
    if (src != nullptr) {
        std::memcpy(dst.data(), src, sizeof(float) * 4 * static_cast<size_t>(count));
    }
}

} // namespace

extern "C" {

void* ref_solver_create(void) { return new physics::FluidSolver(); }

void ref_solver_destroy(void* solver) { delete static_cast<physics::FluidSolver*>(solver); }

int ref_solver_set_state(void* handle, const float* positions, const float* velocities, uint32_t count) {
    auto* solver = static_cast<physics::FluidSolver*>(handle);
    copyIn(solver->positions, positions, count);
    copyIn(solver->velocities, velocities, count);
    solver->nextPositions.assign(count, glm::vec4{0.0F});
    solver->nextVelocities.assign(count, glm::vec4{0.0F});
    solver->previousRendered = solver->positions;
    return SPH_OK;
}

int ref_solver_get_state(void* handle, float* positions, float* velocities) {
    auto* solver = static_cast<physics::FluidSolver*>(handle);
    size_t bytes = sizeof(float) * 4 * solver->positions.size();
    if (positions != nullptr) {
        std::memcpy(positions, solver->positions.data(), bytes);
    }
    if (velocities != nullptr) {
        std::memcpy(velocities, solver->velocities.data(), bytes);
    }
    return SPH_OK;
}

int ref_solver_get_previous(void* handle, float* positions) {
    auto* solver = static_cast<physics::FluidSolver*>(handle);
    std::memcpy(positions, solver->previousParticles().data(), sizeof(float) * 4 * solver->previousParticles().size());
    return SPH_OK;
}

uint32_t ref_solver_count(void* handle) { return static_cast<physics::FluidSolver*>(handle)->particleCount(); }

int ref_solver_emit(void* handle, const sph_params* params, uint32_t count) {
    static_cast<physics::FluidSolver*>(handle)->emit(toReference(*params), count);
    return SPH_OK;
}

int ref_solver_step(void* handle, const sph_params* params, float delta_seconds, uint32_t threads) {
    static_cast<physics::FluidSolver*>(handle)->step(toReference(*params), delta_seconds, jobsFor(threads));
    return SPH_OK;
}

int ref_solver_substep(void* handle, const sph_params* params, float dt, uint32_t threads) {
    static_cast<physics::FluidSolver*>(handle)->substep(toReference(*params), dt, jobsFor(threads));
    return SPH_OK;
}

int ref_solver_keep_rendered(void* handle) {
    static_cast<physics::FluidSolver*>(handle)->keepRendered();
    return SPH_OK;
}

int ref_grid_build(const sph_params* params,
                   const float* positions,
                   uint32_t count,
                   uint32_t* cell_of,
                   uint32_t* cell_counts,
                   uint32_t* cell_particles,
                   uint32_t threads) {
    std::vector<glm::vec4> particles;
    copyIn(particles, positions, count);
    physics::FluidGrid grid;
    grid.build(particles, toReference(*params), jobsFor(threads));
    if (cell_of != nullptr) {
        std::memcpy(cell_of, grid.cellOf.data(), grid.cellOf.size() * sizeof(uint32_t));
    }
    if (cell_counts != nullptr) {
        std::memcpy(cell_counts, grid.cellCounts.data(), grid.cellCounts.size() * sizeof(uint32_t));
    }
    if (cell_particles != nullptr) {
        for (uint32_t b = 0; b < params->lattice[3]; ++b) {
            for (uint32_t k = 0; k < grid.bucketCount(b); ++k) {
                cell_particles[static_cast<size_t>(b) * physics::FLUID_CELL_CAPACITY + k] = grid.particleAt(b, k);
            }
        }
    }
    return SPH_OK;
}

void ref_mc_table(int8_t* out) {
    for (uint32_t code = 0; code < 256; ++code) {
        for (uint32_t i = 0; i < physics::MC_TABLE_WIDTH; ++i) {
            out[code * physics::MC_TABLE_WIDTH + i] = physics::MC_TABLE[code][i];
        }
    }
}

int ref_surface_field(const sph_params* params, const float* positions, uint32_t count, uint32_t resolution,
                      uint32_t threads, float* field) {
    std::vector<glm::vec4> particles;
    copyIn(particles, positions, count);
    std::vector<float> out;
    physics::FluidGrid grid;
    physics::buildFluidField(particles, toReference(*params), resolution, out, grid, jobsFor(threads));
    std::memcpy(field, out.data(), out.size() * sizeof(float));
    return SPH_OK;
}

// Serial (no job system), so that vertices come out in cell order.
int ref_march_field(const float* field, uint32_t resolution, const float origin[3], const float cell[3], float iso,
                    sph_surface_vertex* out, uint32_t capacity, uint32_t* written) {
    uint32_t samples = resolution + 1;
    std::vector<float> values(field, field + static_cast<size_t>(samples) * samples * samples);
    std::vector<physics::SurfaceVertex> vertices(std::max<uint32_t>(capacity, 1));
    uint32_t n = physics::marchFluidField(values, resolution, glm::vec3{origin[0], origin[1], origin[2]},
                                          glm::vec3{cell[0], cell[1], cell[2]}, iso, vertices.data(), capacity,
                                          nullptr);
    for (uint32_t i = 0; i < n; ++i) {
        out[i].position[0] = vertices[i].position.x;
        out[i].position[1] = vertices[i].position.y;
        out[i].position[2] = vertices[i].position.z;
        out[i].normal = vertices[i].normal;
    }
    *written = n;
    return SPH_OK;
}

uint32_t ref_fluid_substeps(const sph_params* params, float delta_seconds) {
    return physics::fluidSubsteps(toReference(*params), delta_seconds);
}

int ref_derive_params(const sph_fluid_settings* settings,
                      const float emitter_world[16],
                      uint32_t particle_count,
                      uint32_t cell_count,
                      sph_params* out) {
    scene::Fluid fluid;
    fluid.emitterHalfExtents =
        glm::vec3{settings->emitter_half_extents[0], settings->emitter_half_extents[1], settings->emitter_half_extents[2]};
    fluid.particleRadius = settings->particle_radius;
    fluid.smoothingRadius = settings->smoothing_radius;
    fluid.restDensity = settings->rest_density;
    fluid.stiffness = settings->stiffness;
    fluid.viscosity = settings->viscosity;
    fluid.containerMin = glm::vec3{settings->container_min[0], settings->container_min[1], settings->container_min[2]};
    fluid.containerMax = glm::vec3{settings->container_max[0], settings->container_max[1], settings->container_max[2]};
    fluid.gravity = glm::vec3{settings->gravity[0], settings->gravity[1], settings->gravity[2]};
    glm::mat4 world;
    for (int c = 0; c < 4; ++c) {
        for (int r = 0; r < 4; ++r) {
            world[c][r] = emitter_world[c * 4 + r];
        }
    }
    scene::Scene scene;
    physics::FluidParams p = physics::deriveFluidParams(fluid, world, particle_count, cell_count, scene);
    std::memset(out, 0, sizeof(*out));
    for (int c = 0; c < 4; ++c) {
        for (int r = 0; r < 4; ++r) {
            out->emitter_world[c * 4 + r] = p.emitterWorld[c][r];
        }
    }
    for (int a = 0; a < 3; ++a) {
        out->emitter_half_extents[a] = p.emitterHalfExtents[a];
        out->container_min[a] = p.containerMin[a];
        out->container_max[a] = p.containerMax[a];
        out->gravity[a] = p.gravity[a];
        out->lattice[a] = p.lattice[a];
    }
    out->emitter_half_extents[3] = p.spacing;
    out->container_min[3] = p.particleRadius;
    out->container_max[3] = p.wallRestitution;
    out->gravity[3] = p.particleMass;
    out->smoothing_radius = p.smoothingRadius;
    out->rest_density = p.restDensity;
    out->stiffness = p.stiffness;
    out->viscosity = p.viscosity;
    out->lattice[3] = p.cellCount;
    return SPH_OK;
}

} // extern "C"
