/*
 * sph_c.h — C ABI of the GB300 SPH fluid step.
 *
 * This is the drop-in boundary for the reference's CPU fluid solver
 * (`physics::FluidSolver`, src/physics/fluid_sph.h:101-127) and for the
 * parameter block its Vulkan twin uploads (`gfx::GpuFluidParams`,
 * src/gfx/fluid.h:81-102). Everything here is plain C: pointers, sizes and
 * status codes. No CUDA or torch type crosses it.
 *
 * Conventions
 *   - Every call returns an `int` status: SPH_OK (0) or a negative
 *     `sph_status`. No call aborts the process.
 *   - Host pointers are owned by the caller. Device buffers are owned by the
 *     context. Particle arrays are the reference's AoS float4 layout:
 *     positions (x, y, z, density) and velocities (vx, vy, vz, pressure),
 *     `4*n` floats each, particles in id order.
 *   - A context owns one CUDA stream. A context is not thread-safe; distinct
 *     contexts are independent.
 *   - Calls that launch work enqueue it on the context stream. Calls that
 *     return host data synchronise that stream first.
 */
#ifndef SPH_C_H
#define SPH_C_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SPH_ABI_VERSION 1

/* Bucket capacity of the hash grid (src/physics/fluid_sph.h:23). */
#define SPH_CELL_CAPACITY 32u
/* Array sizes of the parameter block (fluid_sph.h:22, force_field.h:17). */
#define SPH_MAX_COLLIDERS 8u
#define SPH_MAX_FORCE_FIELDS 8u
/* Longest frame a step catches up on (fluid_sph.h:76). */
#define SPH_MAX_FRAME_STEP (1.0f / 30.0f)

typedef enum sph_status {
    SPH_OK = 0,
    SPH_ERR_INVALID_ARGUMENT = -1,
    SPH_ERR_CAPACITY = -2,
    SPH_ERR_CUDA = -3,
    SPH_ERR_OUT_OF_MEMORY = -4,
    SPH_ERR_UNSUPPORTED = -5,
    SPH_ERR_TIMEOUT = -6,
    SPH_ERR_NO_DEVICE = -7,
    SPH_ERR_NONFINITE = -8
} sph_status;

/* One shape collider; layout of gfx::GpuFluidCollider (fluid.h:50-58). */
typedef struct sph_collider {
    float data0[4];          /* xyz half extents, w radius */
    float inverse_world[16]; /* column-major */
    float world[16];         /* column-major */
    uint32_t type;           /* scene::ColliderShape: 0 sphere, 1 box, 2 plane, 3 cylinder, 4 capsule */
    uint32_t pad[3];
} sph_collider;

/* One force field; layout of gfx::GpuForceField (fluid.h:61-68). */
typedef struct sph_force_field {
    float position_radius[4]; /* xyz centre, w radius (0 = unbounded) */
    float axis_strength[4];   /* xyz direction or axis, w strength */
    float falloff;
    uint32_t type; /* 0 wind, 1 vortex, 2 point */
    uint32_t pad[2];
} sph_force_field;

/*
 * Simulation constants; scalar layout of gfx::GpuFluidParams
 * (fluid.h:81-102), which carries physics::FluidParams (fluid_sph.h:42-67).
 */
typedef struct sph_params {
    float emitter_world[16];       /* column-major mat4 */
    float emitter_half_extents[4]; /* xyz half extents, w lattice spacing */
    float container_min[4];        /* xyz, w particle radius */
    float container_max[4];        /* xyz, w wall restitution */
    float gravity[4];              /* xyz, w particle mass */
    float smoothing_radius;
    float rest_density;
    float stiffness;
    float viscosity;
    uint32_t lattice[4]; /* xyz emit lattice counts, w bucket count (power of two) */
    uint32_t collider_count;
    uint32_t pad0, pad1, pad2;
    sph_collider colliders[SPH_MAX_COLLIDERS];
    uint32_t field_count;
    uint32_t field_pad0, field_pad1, field_pad2;
    sph_force_field fields[SPH_MAX_FORCE_FIELDS];
} sph_params;

/* The physics fields of scene::Fluid (src/scene/scene.h:186-218). */
typedef struct sph_fluid_settings {
    float emitter_half_extents[3];
    float particle_radius;
    float smoothing_radius;
    float rest_density;
    float stiffness;
    float viscosity;
    float container_min[3];
    float container_max[3];
    float gravity[3];
} sph_fluid_settings;

/* Per-substep statistics; FP64 reductions on the device. */
typedef struct sph_stats {
    uint32_t particles;
    uint32_t buckets;
    uint32_t max_bucket_count;  /* largest un-truncated bucket count */
    uint32_t overflow_buckets;  /* buckets holding more than SPH_CELL_CAPACITY */
    uint64_t candidates;        /* neighbour candidates visited by density */
    uint64_t pairs_in_range;    /* candidates with squared distance < h^2 */
    double mean_density;
    double mean_compression;    /* mean over particles of max(0, rho - rho0) / rho0 */
    double max_density;
    double centre_of_mass[3];
    double kinetic_energy;
    uint32_t nonfinite;         /* particles with a non-finite position or velocity */
    uint32_t pad;
} sph_stats;

/* Launch shape of the step; results do not depend on it. */
typedef struct sph_tuning {
    uint32_t radix_bits;       /* digit width of the grid sort, 1..8 */
    uint32_t neighbour_kernel; /* 0: nested per-candidate loops; 1: flat stream + queued pair pass;
                                  2: density records in-range pairs, integrate runs them;
                                  3: as 2, divisions through a shared correctly rounded reciprocal;
                                  4: density stores per-bucket pair masks, integrate expands them;
                                  5: cell-cooperative: the particles of a cell share one candidate list in
                                     shared memory, lanes take candidates (density) and pairs (integrate);
                                  6: the masks of 4; integrate copies every bucket its block visits into
                                     shared memory once and reads the pairs there (Morton or Hilbert order) */
    uint32_t block_size;       /* threads per block of integrate (32..512, multiple of 32; 64/128/256 for 2-4;
                                  128/256 for 6; default 128) */
    uint32_t queue_depth;      /* in-range pairs buffered per thread: 8, 16, 24 or 32 */
    uint32_t schedule;         /* processing order: 0 sorted (bucket) order; 1 (default) Morton order of
                                  the cells; 2 Hilbert order of the cells; orders 1 and 2 are remade every
                                  8 grid builds (every 3 when made by counting: one tank whose cells fit
                                  128 a side; a batch, where 1 and 2 both give each tank's cells in row
                                  order, tank after tank) */
    uint32_t sort;             /* grid sort: 0 three kernels per digit pass (radix_bits wide);
                                  1 one kernel per 8-bit pass, tile offsets from tile digit counts
                                    made by the previous pass (radix_bits unused);
                                  2 (default) counting placement: one atomic place per particle in its
                                    bucket, a scan of the bucket counts, each bucket's 32 smallest ids
                                    put at its front in order with the gather (no radix passes).
                                  The particle sets of the learned form's fallback use sort 1. */
} sph_tuning;

typedef struct sph_ctx sph_ctx;

/* ---- version and diagnostics ---------------------------------------- */

/* ABI version of the loaded library (SPH_ABI_VERSION). */
int sph_abi_version(void);
/* Static, human-readable text for a status code. */
const char* sph_status_string(int status);
/* Text of the last CUDA error a context saw ("" if none). */
const char* sph_last_error(const sph_ctx* ctx);

/* ---- host-side parameter rules (no device needed) -------------------- */

/* physics::deriveFluidParams (fluid_sph.cpp:65-100); no colliders or fields. */
int sph_derive_params(const sph_fluid_settings* settings,
                      const float emitter_world[16],
                      uint32_t particle_count,
                      uint32_t cell_count,
                      sph_params* out);
/* physics::fluidSubsteps (fluid_sph.cpp:128-136). */
int sph_fluid_substeps(const sph_params* params, float delta_seconds, uint32_t* substeps);
/* gfx::cellCountFor (src/gfx/fluid.cpp:50-52): clamp(bit_ceil(2n), 1024, 65536). */
uint32_t sph_cell_count_for(uint32_t particles);
/* Same rule without the 65536 ceiling, for tanks beyond the reference's cap. */
uint32_t sph_cell_count_uncapped(uint32_t particles);

/* ---- context lifetime ------------------------------------------------- */

/* Allocates device state for up to `capacity` particles on `device`. */
int sph_create(const sph_params* params, uint32_t capacity, int device, sph_ctx** out);
int sph_destroy(sph_ctx* ctx);
/* Replaces the constants; the bucket count may change (up to the context's
 * bucket capacity, chosen at create as max(lattice[3], uncapped(capacity))). */
int sph_set_params(sph_ctx* ctx, const sph_params* params);
int sph_particle_count(const sph_ctx* ctx, uint32_t* count);

/* ---- physics::FluidSolver surface ------------------------------------- */

/* FluidSolver::emit (fluid_sph.cpp:138-154), on the device. */
int sph_emit(sph_ctx* ctx, uint32_t count);
/* Uploads `count` particles (host AoS float4). `velocities` may be NULL (zeros). */
int sph_upload(sph_ctx* ctx, const float* positions, const float* velocities, uint32_t count);
/* Downloads the current state (host AoS float4). Either pointer may be NULL. */
int sph_download(sph_ctx* ctx, float* positions, float* velocities);
/* sph_upload + `substeps` substeps of `dt` + sph_download in one call, for
 * a caller that keeps the state on the host: the same results and checks,
 * with the velocity upload overlapping the first substep's grid build. From
 * 2^18 particles (one tank, a curve processing order, neighbour kernel 4, no
 * colliders) the velocities are gathered beside the density pass and the
 * last substep integrates three id ranges in turn (the first half of the
 * ids, then two quarters), downloading each range's rows while the next
 * integrates; one substep then runs as one CUDA graph launch. Page-locked
 * host arrays let the copies run asynchronously.
 * `velocities` may be NULL (zeros); either output may be NULL or alias its
 * input. On SPH_ERR_NONFINITE the outputs are left as they were and the
 * context holds the rejected state, as after a rejected sph_upload.
 * Synchronises. */
int sph_step_host(sph_ctx* ctx, const float* positions, const float* velocities, uint32_t count, float dt,
                  uint32_t substeps, float* positions_out, float* velocities_out);
/* FluidSolver::step (fluid_sph.cpp:311-321): splits the frame with fluidSubsteps. */
int sph_step(sph_ctx* ctx, float delta_seconds);
/* FluidSolver::substep (fluid_sph.cpp:190-309): one grid + density + integrate pass. */
int sph_substep(sph_ctx* ctx, float dt);
/* FluidSolver::keepRendered (fluid_sph.cpp:156-158). */
int sph_keep_rendered(sph_ctx* ctx);
/* FluidSolver::previousParticles (fluid_sph.h:112): host AoS float4. */
int sph_download_previous(sph_ctx* ctx, float* positions);
/* Waits for all work queued on the context stream. */
int sph_synchronize(sph_ctx* ctx);

/* ---- grid of the last substep, in physics::FluidGrid form ------------- */

/*
 * FluidGrid::build output (fluid_sph.cpp:160-188) for the positions the last
 * substep started from: cell_of[n], cell_counts[C] (un-truncated) and
 * cell_particles[C*32] (ids ascending per bucket, first 32 kept; slots past
 * a bucket's count are left untouched). Any pointer may be NULL.
 */
int sph_grid_download(sph_ctx* ctx, uint32_t* cell_of, uint32_t* cell_counts, uint32_t* cell_particles);
/* Builds the grid for the current positions without stepping. */
int sph_grid_build(sph_ctx* ctx);

/*
 * Grid build that allocates nothing. This entry point has no counterpart in
 * the reference. It is for callers that cannot allocate device memory at the
 * point where they build the grid: a render loop that records a frame's GPU
 * work under a fixed device-memory budget (its engine hands all memory to its
 * own allocator up front), or a latency-critical loop that cannot afford the
 * implicit device synchronisation a cudaMalloc may bring.
 *
 * The caller passes device buffers: `positions` (count AoS float4 (x, y, z,
 * w), id order, 16-byte aligned), and receives `cell_of` (count u32: the
 * bucket of each particle), `cell_counts` (C u32: particles per bucket, not
 * truncated) and `cell_particles` (C * 32 u32: the first 32 ids of each
 * bucket, ascending; slots past a bucket's count are left untouched), for
 * C = params->lattice[3] buckets. The u32 arrays must be 4-byte aligned; a
 * misaligned buffer returns SPH_ERR_INVALID_ARGUMENT. Work is enqueued on
 * `stream` (a cudaStream_t, NULL for the legacy default stream) and is
 * complete when that stream reaches it.
 *
 * The sort's scratch is a static device array inside the library, sized for
 * at most SPH_STATIC_MAX_PARTICLES particles and SPH_STATIC_MAX_CELLS buckets
 * (about 1.6 MB, held on every GPU that uses this call until the process
 * exits); larger requests return SPH_ERR_CAPACITY. Every call made outside a
 * stream capture looks the array's device address up (cudaGetSymbolAddress)
 * in the current context, so a context reset or a different current context
 * is picked up; a call on a stream that is being captured reuses the address
 * found by the last uncaptured call on that device, so make one call on each
 * device before capturing it (a captured call without one returns
 * SPH_ERR_CUDA). All calls share the one array, so calls whose work overlaps
 * on the GPU (on different streams, or from different threads) race with each
 * other: serialise them. A CUDA failure returns SPH_ERR_CUDA; this call has
 * no context object, so no error text goes with it.
 */
#define SPH_STATIC_MAX_PARTICLES 65536u
#define SPH_STATIC_MAX_CELLS 65536u
int sph_grid_build_static(const sph_params* params,
                          const void* positions,
                          uint32_t count,
                          void* cell_of,
                          void* cell_counts,
                          void* cell_particles,
                          void* stream);

/* ---- statistics -------------------------------------------------------- */

/* Reduces statistics of the current state (FP64 on the device). */
int sph_stats_compute(sph_ctx* ctx, sph_stats* out);

/* ---- draw instances ------------------------------------------------------
 * The instance writer of the reference's renderer (shaders/fluid_instances.comp,
 * CPU twin src/gfx/fluid.cpp:402-466) into caller-owned device buffers: one
 * gfx::GpuInstance per particle (a sphere scaled by the particle radius at
 * its position, the previous frame's position for motion vectors) and,
 * optionally, one VkAccelerationStructureInstanceKHR-layout record each. */

/* gfx::GpuInstance (src/gfx/geometry.h:98-118), 224 bytes. */
typedef struct sph_instance {
    float model[16];          /* column-major */
    float previous_model[16];
    float normal_matrix[16];
    uint32_t mesh_index;
    uint32_t bucket;
    uint32_t bucket_base;
    uint32_t joint_offset;                   /* NO_JOINTS */
    uint32_t skinned_vertex_offset;          /* NO_SKINNED_VERTICES */
    uint32_t previous_skinned_vertex_offset; /* NO_SKINNED_VERTICES */
    uint32_t skinned_meshlet_offset;
    uint32_t visibility_base;
} sph_instance;

/* VkAccelerationStructureInstanceKHR layout, 64 bytes: a row-major 3x4
 * transform, custom index (24 bits) | mask << 24, SBT offset | flags << 24,
 * acceleration-structure address. */
typedef struct sph_tlas_instance {
    float transform[12];
    uint32_t custom_index_mask;
    uint32_t sbt_offset_flags;
    uint64_t blas;
} sph_tlas_instance;

#define SPH_INSTANCES_RESET_HISTORY 1u /* previous position := current (fresh emit) */
#define SPH_INSTANCES_WRITE_TLAS 2u    /* also write one TLAS record per particle */
#define SPH_INSTANCES_SURFACE_TLAS 4u  /* surface mode: record 0 is the surface, the rest inactive */
#define SPH_NO_JOINTS 0xFFFFFFFFu
#define SPH_FLUID_SURFACE_CUSTOM_INDEX 0x800000u
#define SPH_FLUID_SURFACE_RAY_MASK 0x01u

/* Writes instances[instance_base + i] (and tlas[tlas_base + i]) for every
 * particle, then keeps the current positions as the previous ones
 * (FluidSolver::keepRendered). `instances` and `tlas` are 16-byte aligned
 * device pointers (tlas may be NULL without SPH_INSTANCES_WRITE_TLAS); `blas` is the sphere's
 * (or, in surface mode, the surface's) acceleration-structure address and
 * fluid_index goes into the surface record's custom index. */
int sph_write_instances(sph_ctx* ctx, void* instances, uint32_t instance_base, uint32_t sphere_mesh, void* tlas,
                        uint32_t tlas_base, uint64_t blas, uint32_t fluid_index, uint32_t flags);

/* ---- fluid surface: scalar field + marching cubes ----------------------
 * physics::buildFluidField / physics::marchFluidField
 * (src/physics/marching_cubes.h:39-57, marching_cubes.cpp:312-483) on the
 * device. The field holds (resolution+1)^3 samples, x fastest; its border
 * samples are 0. Vertices come out as triangles in the reference's serial
 * (cell index) order. */

/* Triangle-table width and the largest vertex count one cell emits
 * (MC_TABLE_WIDTH, MC_MAX_TRIANGLES * 3 in marching_cubes.h:19-20). */
#define SPH_MC_TABLE_WIDTH 16u
#define SPH_MC_MAX_CELL_VERTICES 15u
/* Largest resolution the device path accepts (samples = resolution + 1 per
 * axis); 15 vertices for each of 640^3 cells still fit a 32-bit count. */
#define SPH_SURFACE_MAX_RESOLUTION 640u

/* physics::SurfaceVertex (marching_cubes.h:29-34): position and an
 * octahedral-packed unit normal (asset::packUnitVector). */
typedef struct sph_surface_vertex {
    float position[3];
    uint32_t normal;
} sph_surface_vertex;

/* The marching-cubes case table (256 x SPH_MC_TABLE_WIDTH edge indices, -1
 * ends a case) the device uses; it is generated from the face-contour rule
 * the reference documents for MC_TABLE (marching_cubes.cpp:18-24). */
int sph_surface_table(int8_t out[256 * 16]);
/* buildFluidField on the context's particles and constants: rebuilds the
 * grid from the current positions (afterwards sph_grid_download returns that
 * grid), then samples the field into a context-owned device buffer. */
int sph_surface_field(sph_ctx* ctx, uint32_t resolution);
/* Copies the last field to the host ((resolution+1)^3 floats). */
int sph_surface_field_download(sph_ctx* ctx, float* field);
/* marchFluidField on the context's last field with origin = container_min and
 * cell = (container_max - container_min) / resolution, into a context-owned
 * buffer of `capacity` vertices; *written is the vertex count (<= capacity;
 * 0 if capacity < 3). */
int sph_surface_march(sph_ctx* ctx, float iso, uint32_t capacity, uint32_t* written);
/* Copies the first `count` vertices of the last march to the host. */
int sph_surface_vertices_download(sph_ctx* ctx, sph_surface_vertex* out, uint32_t count);
/* Device pointers of the context's field and vertex buffers (NULL until made). */
int sph_surface_device(sph_ctx* ctx, const float** field, const sph_surface_vertex** vertices);
/* marchFluidField on any host field, on `device`: host in, host out. */
int sph_march_field(const float* field,
                    uint32_t resolution,
                    const float origin[3],
                    const float cell[3],
                    float iso,
                    sph_surface_vertex* out,
                    uint32_t capacity,
                    uint32_t* written,
                    int device);

/* ---- device-resident access (for callers that keep data in HBM) ------- */

/* The context's cudaStream_t, as an opaque pointer. */
int sph_stream(sph_ctx* ctx, void** stream);
/* Device pointers to the current positions and velocities (AoS float4,
 * id order). They change after every substep (ping-pong); fetch again. */
int sph_device_state(sph_ctx* ctx, void** positions, void** velocities);
/* Enqueues `substeps` substeps of `dt` without host synchronisation. */
int sph_run(sph_ctx* ctx, float dt, uint32_t substeps);
/* Runs `substeps` substeps without the CUDA graph and adds the device time of
 * each phase, measured with CUDA events on the context stream, to
 * phase_ms[0..5]: keys, radix sort, bounds + gather, density, integrate, and
 * shapes (the force-field and collider passes; 0 without fields and
 * colliders). Under sort 2 the keys phase holds the counting placement up to
 * the scan and placement, the sort phase nothing, and bounds + gather the
 * final ordering with the gather. Synchronises. Results are identical to
 * sph_run. */
#define SPH_PROFILE_PHASES 6
int sph_profile_substeps(sph_ctx* ctx, float dt, uint32_t substeps, double* phase_ms);
/* Reads / replaces the launch shape (an autotuner's knobs). */
int sph_get_tuning(const sph_ctx* ctx, sph_tuning* out);
int sph_set_tuning(sph_ctx* ctx, const sph_tuning* tuning);
/* Diagnostic: counts, over `count` generated (x, y), the quotients where
 * division through a correctly rounded reciprocal (the integrate pass of
 * neighbour_kernel 3) differs from IEEE x / y. mode 0: every divisor mantissa
 * in [1, 2); mode 1: random signs, mantissas and exponents 2^-60..2^60; mode 6:
 * y = the float with the seed's low 32 bits and x `count` consecutive floats
 * from the one with its high 32 bits (an exhaustive sweep of one divisor). */
int sph_selftest_division(sph_ctx* ctx, uint64_t seed, uint64_t count, int mode, uint64_t* mismatches);
/* Number of kernel launches one substep enqueues. */
int sph_launches_per_substep(const sph_ctx* ctx, uint32_t* launches);
/* Kernels the context has launched through sph_run / sph_step (the substep
 * graph's kernels) and through the processing-order remakes of every path,
 * counted as they are enqueued: the difference across a region of sph_run
 * calls is the number of kernels that region ran. */
int sph_kernels_launched(const sph_ctx* ctx, uint64_t* kernels);
/* Bytes of device memory the context holds. */
int sph_device_bytes(const sph_ctx* ctx, uint64_t* bytes);

/* Times candidate launch shapes (neighbour kernel, block size, processing
 * order, radix digit width) on the current state, which is restored
 * afterwards, and keeps the fastest. Results are bit-identical for every
 * shape. */
int sph_autotune(sph_ctx* ctx, float dt, uint32_t substeps_per_trial, sph_tuning* best, float* best_ms);

/* ---- batched tanks ------------------------------------------------------
 *
 * Many independent fluids ("tanks", each a physics::FluidSolver) advanced by
 * the same kernel launches: one CUDA graph launch per substep covers every
 * tank. Tank t has its own sph_params (container, lattice, bucket count) and a
 * particle count fixed at create. There is no reference counterpart beyond
 * the per-tank FluidSolver semantics (fluid_sph.cpp:190-321), which each tank
 * keeps bit for bit. */
#define SPH_ALL_TANKS 0xFFFFFFFFu
typedef struct sph_batch sph_batch;

int sph_batch_create(const sph_params* params, const uint32_t* counts, uint32_t tanks, int device, sph_batch** out);
int sph_batch_destroy(sph_batch* batch);
const char* sph_batch_last_error(const sph_batch* batch);
int sph_batch_tank_count(const sph_batch* batch, uint32_t* tanks);
/* Particles of one tank, or of all tanks with SPH_ALL_TANKS. */
int sph_batch_particle_count(const sph_batch* batch, uint32_t tank, uint32_t* count);
/* Host AoS float4 arrays of the tank's fixed particle count; velocities may be NULL. */
int sph_batch_upload(sph_batch* batch, uint32_t tank, const float* positions, const float* velocities);
int sph_batch_download(sph_batch* batch, uint32_t tank, float* positions, float* velocities);
/* FluidSolver::emit for one tank. */
int sph_batch_emit(sph_batch* batch, uint32_t tank);
/* Tanks with active[t] == 0 keep their state through later substeps. */
int sph_batch_set_active(sph_batch* batch, const uint8_t* active);
/* `substeps` substeps of `dt` for every active tank. While the active tanks
 * hold at most half the particles, the grid is built over their particles
 * alone (same bits, less work). */
int sph_batch_run(sph_batch* batch, float dt, uint32_t substeps);
/* Tank t runs substeps[t] substeps of dt[t]; tanks done early sit out. */
int sph_batch_run_per_tank(sph_batch* batch, const float* dt, const uint32_t* substeps);
/* FluidSolver::step for every tank (each with its own fluidSubsteps). */
int sph_batch_step(sph_batch* batch, float delta_seconds);
/* FP64 statistics of every tank into out[tanks]. */
int sph_batch_stats(sph_batch* batch, sph_stats* out);
int sph_batch_synchronize(sph_batch* batch);
int sph_batch_stream(sph_batch* batch, void** stream);
int sph_batch_get_tuning(const sph_batch* batch, sph_tuning* out);
int sph_batch_set_tuning(sph_batch* batch, const sph_tuning* tuning);
int sph_batch_autotune(sph_batch* batch, float dt, uint32_t substeps_per_trial, sph_tuning* best, float* best_ms);
/* sph_profile_substeps for the whole batch: SPH_PROFILE_PHASES totals. */
int sph_batch_profile_substeps(sph_batch* batch, float dt, uint32_t substeps, double* phase_ms);
int sph_batch_launches_per_substep(const sph_batch* batch, uint32_t* launches);
int sph_batch_device_bytes(const sph_batch* batch, uint64_t* bytes);

/* ---- learned acceleration correction (MLP) ------------------------------
 *
 * No counterpart in the reference. A 32 -> 128 -> 128 -> 3 MLP with GELU
 * (erf form), BF16 weights and FP32 accumulation; forward on the tensor cores
 * (tcgen05), backward and Adam (src/gfx/neural_math.cpp:1177-1208) on the CUDA
 * cores. Inputs are 32 FP32 features per particle (sph_batch_learned_sample
 * documents them); outputs are accelerations (m/s^2) in an n x 4 array
 * (xyz, w = 0). Feature and target arrays are device pointers. */
#define SPH_MLP_INPUTS 32
#define SPH_MLP_HIDDEN 128
#define SPH_MLP_OUTPUTS 3
/* FP32 parameter vector: W1[128][32], b1[128], W2[128][128], b2[128], W3[3][128], b3[3]. */
#define SPH_MLP_PARAMS 21123
typedef struct sph_mlp sph_mlp;

/* He-normal weights from a seeded splitmix64 stream, zero biases. */
int sph_mlp_create(int device, uint64_t seed, sph_mlp** out);
int sph_mlp_destroy(sph_mlp* mlp);
const char* sph_mlp_last_error(const sph_mlp* mlp);
int sph_mlp_get_params(sph_mlp* mlp, float* params);
/* Replaces the FP32 parameters (BF16 copies refreshed, Adam state reset). */
int sph_mlp_set_params(sph_mlp* mlp, const float* params);
/* Inputs are normalised as (f - mean) / std; outputs are network * scale. */
int sph_mlp_set_normalisation(sph_mlp* mlp, const float* feature_mean, const float* feature_std,
                              const float* output_scale);
int sph_mlp_get_normalisation(sph_mlp* mlp, float* feature_mean, float* feature_std, float* output_scale);
/* accel[n][4] = MLP(features[n][32]). With stream == NULL the call runs on
 * the model's stream and synchronises; otherwise it is enqueued on `stream`. */
int sph_mlp_forward(sph_mlp* mlp, const void* features, uint32_t count, void* accel, void* stream);
/* Gradient of the mean squared error between the normalised output and
 * targets[n][3] / output_scale, into grads[SPH_MLP_PARAMS] (host); no update. */
int sph_mlp_gradients(sph_mlp* mlp, const void* features, const void* targets, uint32_t count, float* grads,
                      float* loss);
int sph_mlp_set_adam(sph_mlp* mlp, float beta1, float beta2, float epsilon);
/* One Adam step on a batch; loss (host, may be NULL) is the batch's loss. */
int sph_mlp_train_step(sph_mlp* mlp, const void* features, const void* targets, uint32_t count, float learning_rate,
                       float* loss);
int sph_mlp_stream(sph_mlp* mlp, void** stream);
/* Learned steps with this model take each tank's mean correction off along
 * the axes set in `axes` (bit 0 x, 1 y, 2 z; 0, the default, keeps it), so
 * the correction exerts no net force on a tank along them. No counterpart in
 * the reference (it has no learned fluid path). */
int sph_mlp_set_net_force_free(sph_mlp* mlp, uint32_t axes);
/* One Adam step with a gradient supplied by the caller (host, SPH_MLP_PARAMS
 * floats), e.g. the average of several GPUs' sph_mlp_gradients in
 * data-parallel training. No counterpart in the reference (it has no learned
 * fluid path); the update rule is adamStep (src/gfx/neural_math.cpp:1177-1208). */
int sph_mlp_apply_gradients(sph_mlp* mlp, const float* grads, float learning_rate);
/* Diagnostic: largest |erf(x) - erff(x)| of the forward pass's erf
 * (tanh(a u + b u^3), u = sqrt(2) x, the approximation behind the tanh form
 * of GELU, with the hardware tanh) over `count` points on [-6, 6]. */
int sph_mlp_selftest_erf(sph_mlp* mlp, uint32_t count, float* max_abs_error);
/* Diagnostic of the bounded device waits: one block waits on an mbarrier
 * with at most `polls` tries, as the forward pass waits for its tensor-core
 * work; the barrier is arrived at only when `arrive` is nonzero. Returns
 * SPH_OK when the wait completed and SPH_ERR_TIMEOUT when it gave up; either
 * way the context stays usable. No counterpart in the reference (its GPU
 * failure path is a fatal error, src/gfx/fluid.cpp:95-100). */
int sph_mlp_selftest_wait(sph_mlp* mlp, uint32_t polls, int arrive);

/* Learned coarse substeps (no counterpart in the reference): the plain SPH
 * force as in sph_step, plus the MLP's acceleration correction, then the
 * plain velocity update, speed clamp and walls. mlp == NULL runs the same
 * path with a zero correction, which is bit-identical to the plain substep. */
int sph_run_learned(sph_ctx* ctx, float dt, uint32_t substeps, const sph_mlp* mlp);
int sph_batch_run_learned(sph_batch* batch, float dt, uint32_t substeps, const sph_mlp* mlp);
/* The 32 correction features of every particle of the current state (device
 * array, all tanks, id order, n x 32 floats) for a substep of length dt; the
 * state does not change. Feature definitions: csrc/sph_forces.cu. */
int sph_batch_learned_features(sph_batch* batch, float dt, void* features);
/* The acceleration correction a learned substep of length dt would add, from
 * the current state (device array, float4 per particle, id order; the MLP's
 * scaled output before any net-force removal): the learned step's own path
 * (features written as BF16 input tiles, the forward pass over them). Every
 * tank must be active. The state does not change. */
int sph_batch_learned_correction(sph_batch* batch, float dt, const sph_mlp* mlp, void* correction);
/* SPH_ERR_TIMEOUT if a tensor-core completion wait gave up since the last
 * check (the step's results are then not valid). Synchronises. */
int sph_batch_learned_check(sph_batch* batch);
/* Saves (save != 0) or restores the whole particle state in device memory,
 * in slot 0 or 1; sph_batch_restore_tanks copies back only the tanks with
 * which[t] != 0. */
int sph_batch_snapshot(sph_batch* batch, uint32_t slot, int save);
int sph_batch_restore_tanks(sph_batch* batch, uint32_t slot, const uint8_t* which);
/* Device pointers to all tanks' state (AoS float4, id order); tank t starts
 * at particle sph_batch_tank_offset(t). */
int sph_batch_device_state(sph_batch* batch, void** positions, void** velocities);
int sph_batch_tank_offset(const sph_batch* batch, uint32_t tank, uint32_t* first);
/* Copies the whole state (id order, AoS float4) into caller device buffers,
 * enqueued on the batch's stream; either pointer may be NULL. */
int sph_batch_copy_state(sph_batch* batch, void* positions, void* velocities);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* SPH_C_H */
