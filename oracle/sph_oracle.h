/*
 * sph_oracle.h — CPU oracle of the reference's SPH fluid step.
 *
 * TEST INFRASTRUCTURE ONLY. This library is the checker that the CUDA path
 * is compared against (and the CPU baseline that bench.py times beside it).
 * Nothing in the product path links, loads or calls it.
 *
 * It restates, expression by expression, the reference's CPU solver:
 *   src/physics/spatial_hash.h:12-20      spatialCell / spatialHash
 *   src/physics/fluid_sph.cpp:24-46        poly6 / spikyGradient / viscosityLaplacian
 *   src/physics/fluid_sph.cpp:65-100       deriveFluidParams
 *   src/physics/fluid_sph.cpp:128-136      fluidSubsteps
 *   src/physics/fluid_sph.cpp:138-154      FluidSolver::emit
 *   src/physics/fluid_sph.cpp:160-188      FluidGrid::build
 *   src/physics/fluid_sph.cpp:190-309      FluidSolver::substep
 *   src/physics/fluid_sph.cpp:311-321      FluidSolver::step
 *   src/physics/force_field.h:31-70        forceFieldsAcceleration
 *   src/physics/collider_shapes.h:27-134   closestOnColliderLocal (shape colliders)
 *   src/physics/marching_cubes.cpp:300-483 buildFluidField / marchFluidField (serial order)
 *   src/asset/vertex_pack.h:20-51         packUnitVector
 *   src/core/job_system.cpp:80-117         parallelFor chunking (granularity 256)
 * and is pinned against the unmodified reference sources compiled here
 * (oracle/ref, output in oracle/_ref) by tests/test_oracle_vs_reference.py.
 */
#ifndef SPH_ORACLE_H
#define SPH_ORACLE_H

#include <stdint.h>

#include "../include/sph_c.h"

#ifdef __cplusplus
extern "C" {
#endif

int oracle_abi(void);
uint32_t oracle_spatial_hash(int32_t cx, int32_t cy, int32_t cz, uint32_t cell_count);
void oracle_spatial_cell(const float position[3], float cell_size, int32_t out[3]);

int oracle_derive_params(const sph_fluid_settings* settings,
                         const float emitter_world[16],
                         uint32_t particle_count,
                         uint32_t cell_count,
                         sph_params* out);
uint32_t oracle_fluid_substeps(const sph_params* params, float delta_seconds);
void oracle_emit(const sph_params* params, uint32_t count, float* positions, float* velocities);

/* FluidGrid::build. cell_particles holds cell_count*32 slots. */
int oracle_grid_build(const sph_params* params,
                      const float* positions,
                      uint32_t count,
                      uint32_t* cell_of,
                      uint32_t* cell_counts,
                      uint32_t* cell_particles,
                      uint32_t threads);

/* One substep in place. threads = 0 or 1 runs serially. */
int oracle_substep(const sph_params* params, float* positions, float* velocities, uint32_t count, float dt, uint32_t threads);
/* FluidSolver::step in place. */
int oracle_step(const sph_params* params,
                float* positions,
                float* velocities,
                uint32_t count,
                float delta_seconds,
                uint32_t threads);
/* Density pass alone (writes positions[i].w and velocities[i].w in place). */
int oracle_density(const sph_params* params, float* positions, float* velocities, uint32_t count, uint32_t threads);

/* Candidates visited by the density loop (P) and those with r^2 < h^2 (Q). */
int oracle_pair_counts(const sph_params* params,
                       const float* positions,
                       uint32_t count,
                       uint64_t* candidates,
                       uint64_t* in_range,
                       uint32_t threads);

/* FP64 statistics of a state (same definitions as sph_stats). */
int oracle_stats(const sph_params* params, const float* positions, const float* velocities, uint32_t count, sph_stats* out);

/* Worker threads the host offers. */
/* gfx::FluidSimulator's CPU instance writer (src/gfx/fluid.cpp:402-466):
 * per particle one instance record (model = scale(translate(I, p), r); the
 * previous model from `prev` unless SPH_INSTANCES_RESET_HISTORY; identity
 * normal matrix; `sphere_mesh`; no joints or skinned vertices) and, with
 * SPH_INSTANCES_WRITE_TLAS, its acceleration-structure record (row-major 3x4
 * of the model, custom index = slot & 0xFFFFFF, mask 0xFF, `blas`); with
 * SPH_INSTANCES_SURFACE_TLAS as well, record 0 is the surface and the others
 * are zero. Positions and previous positions are AoS float4. */
int oracle_write_instances(const float* pos, const float* prev, uint32_t n, float radius, sph_instance* instances,
                           uint32_t instance_base, uint32_t sphere_mesh, sph_tlas_instance* tlas, uint32_t tlas_base,
                           uint64_t blas, uint32_t fluid_index, uint32_t flags, uint32_t threads);
uint32_t oracle_hardware_threads(void);

void oracle_mc_table(int8_t* out);
int oracle_surface_field(const sph_params* params, const float* positions, uint32_t count, uint32_t resolution,
                         uint32_t threads, float* field);
int oracle_march_field(const float* field, uint32_t resolution, const float origin[3], const float cell[3], float iso,
                       sph_surface_vertex* out, uint32_t capacity, uint32_t* written);

#ifdef __cplusplus
}
#endif

#endif
