// sph_capi.cu — the extern "C" entry points of include/sph_c.h.
//
// Each entry point checks its arguments, forwards to the Engine and returns
// a status code; none aborts. The context is the GPU counterpart of one
// physics::FluidSolver (src/physics/fluid_sph.h:101-127).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/sph_c.h"
#include "sph_engine.h"
#include "sph_mlp.cuh"

struct sph_ctx {
    sph::Engine engine;
};

struct sph_batch {
    sph::Engine engine;
};

namespace {

uint32_t bit_ceil(uint32_t x) {
    if (x <= 1) {
        return 1;
    }
    uint32_t v = 1;
    while (v < x && v != 0x80000000u) {
        v <<= 1;
    }
    return v;
}

void to_api(const sph::TuneChoice& c, sph_tuning* out) {
    out->radix_bits = c.radix_bits;
    out->neighbour_kernel = c.tuning.variant;
    out->block_size = c.tuning.block;
    out->queue_depth = c.tuning.queue;
    out->schedule = c.schedule;
    out->sort = c.counting ? 2u : (c.onesweep ? 1u : 0u);
}

int autotune(sph::Engine& engine, float dt, uint32_t substeps, sph_tuning* best, float* best_ms) {
    if (best == nullptr) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    sph::TuneChoice choice;
    int status = engine.autotune(dt, substeps, &choice, nullptr);
    if (status == SPH_OK) {
        to_api(choice, best);
        if (best_ms != nullptr) {
            *best_ms = choice.ms;
        }
    }
    return status;
}

}  // namespace

extern "C" {

int sph_abi_version(void) { return SPH_ABI_VERSION; }

const char* sph_status_string(int status) {
    switch (status) {
    case SPH_OK:
        return "ok";
    case SPH_ERR_INVALID_ARGUMENT:
        return "invalid argument";
    case SPH_ERR_CAPACITY:
        return "capacity exceeded";
    case SPH_ERR_CUDA:
        return "CUDA error";
    case SPH_ERR_OUT_OF_MEMORY:
        return "out of device memory";
    case SPH_ERR_UNSUPPORTED:
        return "unsupported configuration";
    case SPH_ERR_TIMEOUT:
        return "device wait timed out";
    case SPH_ERR_NO_DEVICE:
        return "no CUDA device";
    case SPH_ERR_NONFINITE:
        return "non-finite input";
    default:
        return "unknown status";
    }
}

const char* sph_last_error(const sph_ctx* ctx) { return ctx == nullptr ? "" : ctx->engine.last_error(); }

// deriveFluidParams (src/physics/fluid_sph.cpp:65-100), scene-free.
int sph_derive_params(const sph_fluid_settings* settings,
                      const float emitter_world[16],
                      uint32_t particle_count,
                      uint32_t cell_count,
                      sph_params* out) {
    if (settings == nullptr || emitter_world == nullptr || out == nullptr) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    std::memset(out, 0, sizeof(*out));
    float spacing = settings->particle_radius * 2.0F;
    std::memcpy(out->emitter_world, emitter_world, sizeof(out->emitter_world));
    for (int a = 0; a < 3; ++a) {
        out->emitter_half_extents[a] = settings->emitter_half_extents[a];
        out->container_min[a] = settings->container_min[a];
        out->container_max[a] = settings->container_max[a];
        out->gravity[a] = settings->gravity[a];
    }
    out->emitter_half_extents[3] = spacing;
    out->container_min[3] = settings->particle_radius;
    out->container_max[3] = 0.3F;
    out->gravity[3] = settings->rest_density * spacing * spacing * spacing;
    out->smoothing_radius = std::max(settings->smoothing_radius, spacing);
    out->rest_density = settings->rest_density;
    out->stiffness = settings->stiffness;
    out->viscosity = settings->viscosity;
    auto along = [spacing](float half) {
        return std::max(1U, static_cast<uint32_t>(std::floor(half * 2.0F / spacing)));
    };
    uint32_t nx = along(settings->emitter_half_extents[0]);
    uint32_t ny = along(settings->emitter_half_extents[1]);
    out->lattice[0] = nx;
    out->lattice[1] = ny;
    out->lattice[2] = std::max(1U, (particle_count + nx * ny - 1) / (nx * ny));
    out->lattice[3] = cell_count;
    return SPH_OK;
}

int sph_fluid_substeps(const sph_params* params, float delta_seconds, uint32_t* substeps) {
    if (params == nullptr || substeps == nullptr) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    *substeps = sph::fluid_substeps(*params, delta_seconds);
    return SPH_OK;
}

uint32_t sph_cell_count_for(uint32_t particles) {
    return std::clamp<uint32_t>(bit_ceil(std::max(particles, 1U) * 2), 1024, 65536);
}

uint32_t sph_cell_count_uncapped(uint32_t particles) {
    return std::max<uint32_t>(bit_ceil(std::max(particles, 1U) * 2), 1024);
}

int sph_create(const sph_params* params, uint32_t capacity, int device, sph_ctx** out) {
    if (params == nullptr || out == nullptr || capacity == 0) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    *out = nullptr;
    sph_ctx* ctx = new (std::nothrow) sph_ctx();
    if (ctx == nullptr) {
        return SPH_ERR_OUT_OF_MEMORY;
    }
    int status = ctx->engine.init(device, {*params}, {capacity});
    if (status != SPH_OK) {
        delete ctx;
        return status;
    }
    *out = ctx;
    return SPH_OK;
}

int sph_destroy(sph_ctx* ctx) {
    delete ctx;
    return SPH_OK;
}

int sph_set_params(sph_ctx* ctx, const sph_params* params) {
    if (ctx == nullptr || params == nullptr) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    return ctx->engine.set_params(0, *params);
}

int sph_particle_count(const sph_ctx* ctx, uint32_t* count) {
    if (ctx == nullptr || count == nullptr) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    *count = ctx->engine.count(0);
    return SPH_OK;
}

int sph_emit(sph_ctx* ctx, uint32_t count) {
    if (ctx == nullptr) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    return ctx->engine.emit(0, count);
}

int sph_upload(sph_ctx* ctx, const float* positions, const float* velocities, uint32_t count) {
    if (ctx == nullptr) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    return ctx->engine.upload(0, positions, velocities, count);
}

int sph_step_host(sph_ctx* ctx, const float* positions, const float* velocities, uint32_t count, float dt,
                  uint32_t substeps, float* positions_out, float* velocities_out) {
    if (ctx == nullptr) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    return ctx->engine.step_host(positions, velocities, count, dt, substeps, positions_out, velocities_out);
}

int sph_download(sph_ctx* ctx, float* positions, float* velocities) {
    if (ctx == nullptr) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    return ctx->engine.download(0, positions, velocities);
}

// FluidSolver::step (fluid_sph.cpp:311-321).
int sph_step(sph_ctx* ctx, float delta_seconds) {
    if (ctx == nullptr || std::isnan(delta_seconds)) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    if (ctx->engine.count(0) == 0 || delta_seconds <= 0.0F) {
        return SPH_OK;
    }
    uint32_t substeps = sph::fluid_substeps(ctx->engine.params(0), delta_seconds);
    float frame_step = std::min(delta_seconds, SPH_MAX_FRAME_STEP);
    float dt = frame_step / static_cast<float>(substeps);
    return ctx->engine.run(dt, substeps);
}

int sph_substep(sph_ctx* ctx, float dt) {
    if (ctx == nullptr) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    return ctx->engine.run(dt, 1);
}

int sph_write_instances(sph_ctx* ctx, void* instances, uint32_t instance_base, uint32_t sphere_mesh, void* tlas,
                        uint32_t tlas_base, uint64_t blas, uint32_t fluid_index, uint32_t flags) {
    if (ctx == nullptr) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    return ctx->engine.write_instances(static_cast<sph_instance*>(instances), instance_base, sphere_mesh,
                                       static_cast<sph_tlas_instance*>(tlas), tlas_base, blas, fluid_index, flags);
}

int sph_keep_rendered(sph_ctx* ctx) {
    if (ctx == nullptr) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    return ctx->engine.keep_rendered();
}

int sph_download_previous(sph_ctx* ctx, float* positions) {
    if (ctx == nullptr) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    return ctx->engine.download_previous(0, positions);
}

int sph_synchronize(sph_ctx* ctx) {
    if (ctx == nullptr) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    return ctx->engine.synchronize();
}

int sph_grid_download(sph_ctx* ctx, uint32_t* cell_of, uint32_t* cell_counts, uint32_t* cell_particles) {
    if (ctx == nullptr) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    return ctx->engine.grid_download(0, cell_of, cell_counts, cell_particles);
}

int sph_grid_build(sph_ctx* ctx) {
    if (ctx == nullptr) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    return ctx->engine.build_grid();
}

int sph_surface_table(int8_t out[256 * 16]) {
    if (out == nullptr) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    std::memcpy(out, sph::surface::case_table(), 256 * SPH_MC_TABLE_WIDTH);
    return SPH_OK;
}

int sph_surface_field(sph_ctx* ctx, uint32_t resolution) {
    if (ctx == nullptr) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    return ctx->engine.surface_field(0, resolution);
}

int sph_surface_field_download(sph_ctx* ctx, float* field) {
    if (ctx == nullptr) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    return ctx->engine.surface_field_download(field);
}

int sph_surface_march(sph_ctx* ctx, float iso, uint32_t capacity, uint32_t* written) {
    if (ctx == nullptr) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    return ctx->engine.surface_march(iso, capacity, written);
}

int sph_surface_vertices_download(sph_ctx* ctx, sph_surface_vertex* out, uint32_t count) {
    if (ctx == nullptr) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    return ctx->engine.surface_vertices_download(out, count);
}

int sph_surface_device(sph_ctx* ctx, const float** field, const sph_surface_vertex** vertices) {
    if (ctx == nullptr) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    if (field != nullptr) {
        *field = ctx->engine.surface_field_device();
    }
    if (vertices != nullptr) {
        *vertices = ctx->engine.surface_vertices_device();
    }
    return SPH_OK;
}

int sph_march_field(const float* field, uint32_t resolution, const float origin[3], const float cell[3], float iso,
                    sph_surface_vertex* out, uint32_t capacity, uint32_t* written, int device) {
    if (field == nullptr || origin == nullptr || cell == nullptr || written == nullptr || resolution == 0 ||
        resolution > SPH_SURFACE_MAX_RESOLUTION || (out == nullptr && capacity > 0)) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    *written = 0;
    if (capacity < 3) {
        return SPH_OK;
    }
    int devices = 0;
    if (cudaGetDeviceCount(&devices) != cudaSuccess || devices == 0) {
        cudaGetLastError();
        return SPH_ERR_NO_DEVICE;
    }
    if (device < 0 || device >= devices || cudaSetDevice(device) != cudaSuccess) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    const size_t samples = resolution + 1ull;
    const size_t field_bytes = samples * samples * samples * sizeof(float);
    const uint32_t tiles = sph::surface::march_tiles(resolution);
    float* d_field = nullptr;
    sph_surface_vertex* d_out = nullptr;
    uint8_t* d_codes = nullptr;
    uint32_t* d_tiles = nullptr;
    cudaStream_t stream = nullptr;
    uint32_t result[2] = {0, 0};
    cudaError_t err = cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking);
    if (err == cudaSuccess) err = cudaMalloc(&d_field, field_bytes);
    if (err == cudaSuccess) err = cudaMalloc(&d_out, static_cast<size_t>(capacity) * sizeof(sph_surface_vertex));
    if (err == cudaSuccess) err = cudaMalloc(&d_codes, static_cast<size_t>(resolution) * resolution * resolution);
    if (err == cudaSuccess) err = cudaMalloc(&d_tiles, (2 * static_cast<size_t>(tiles) + 2) * sizeof(uint32_t));
    if (err == cudaSuccess) err = cudaMemcpyAsync(d_field, field, field_bytes, cudaMemcpyHostToDevice, stream);
    if (err == cudaSuccess) {
        sph::surface::MarchGeom g{};
        for (int a = 0; a < 3; ++a) {
            g.origin[a] = origin[a];
            g.cell[a] = cell[a];
        }
        g.iso = iso;
        g.resolution = resolution;
        sph::surface::MarchScratch scratch{d_codes, d_tiles, d_tiles + tiles, d_tiles + 2 * static_cast<size_t>(tiles) + 1};
        err = sph::surface::launch_march(d_field, g, capacity, scratch, d_out, stream);
        if (err == cudaSuccess) err = cudaMemcpyAsync(&result[0], scratch.offsets + tiles, sizeof(uint32_t),
                                                      cudaMemcpyDeviceToHost, stream);
        if (err == cudaSuccess) err = cudaMemcpyAsync(&result[1], scratch.limit, sizeof(uint32_t),
                                                      cudaMemcpyDeviceToHost, stream);
        if (err == cudaSuccess) err = cudaStreamSynchronize(stream);
        if (err == cudaSuccess) {
            *written = std::min(result[0], result[1]);
            err = cudaMemcpy(out, d_out, static_cast<size_t>(*written) * sizeof(sph_surface_vertex),
                             cudaMemcpyDeviceToHost);
        }
    }
    if (stream != nullptr) {
        cudaStreamSynchronize(stream);
        cudaStreamDestroy(stream);
    }
    cudaFree(d_field);
    cudaFree(d_out);
    cudaFree(d_codes);
    cudaFree(d_tiles);
    if (err != cudaSuccess) {
        cudaGetLastError();
        *written = 0;
        return err == cudaErrorMemoryAllocation ? SPH_ERR_OUT_OF_MEMORY : SPH_ERR_CUDA;
    }
    return SPH_OK;
}

int sph_stats_compute(sph_ctx* ctx, sph_stats* out) {
    if (ctx == nullptr || out == nullptr) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    return ctx->engine.stats(0, out, true);
}

int sph_stream(sph_ctx* ctx, void** stream) {
    if (ctx == nullptr || stream == nullptr) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    *stream = static_cast<void*>(ctx->engine.stream());
    return SPH_OK;
}

int sph_device_state(sph_ctx* ctx, void** positions, void** velocities) {
    if (ctx == nullptr) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    if (positions != nullptr) {
        *positions = ctx->engine.positions();
    }
    if (velocities != nullptr) {
        *velocities = ctx->engine.velocities();
    }
    return SPH_OK;
}

int sph_run(sph_ctx* ctx, float dt, uint32_t substeps) {
    if (ctx == nullptr) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    return ctx->engine.run(dt, substeps);
}

int sph_profile_substeps(sph_ctx* ctx, float dt, uint32_t substeps, double* phase_ms) {
    if (ctx == nullptr) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    return ctx->engine.profile(dt, substeps, phase_ms);
}

int sph_get_tuning(const sph_ctx* ctx, sph_tuning* out) {
    if (ctx == nullptr || out == nullptr) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    const sph::NeighbourTuning& t = ctx->engine.tuning();
    out->radix_bits = ctx->engine.radix_bits();
    out->neighbour_kernel = t.variant;
    out->block_size = t.block;
    out->queue_depth = t.queue;
    out->schedule = ctx->engine.schedule_on();
    out->sort = ctx->engine.counting_on() ? 2u : (ctx->engine.onesweep_on() ? 1u : 0u);
    return SPH_OK;
}

int sph_set_tuning(sph_ctx* ctx, const sph_tuning* tuning) {
    if (ctx == nullptr || tuning == nullptr) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    sph::NeighbourTuning t;
    t.variant = tuning->neighbour_kernel;
    t.block = tuning->block_size;
    t.queue = tuning->queue_depth;
    if (tuning->schedule > 2 || tuning->sort > 2) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    int status = ctx->engine.set_tuning(t);
    if (status != SPH_OK) {
        return status;
    }
    status = ctx->engine.set_schedule(tuning->schedule);
    if (status != SPH_OK) {
        return status;
    }
    status = ctx->engine.set_onesweep(tuning->sort != 0);
    if (status == SPH_OK) {
        status = ctx->engine.set_counting(tuning->sort == 2);
    }
    if (status != SPH_OK) {
        return status;
    }
    return ctx->engine.set_radix_bits(tuning->radix_bits);
}

int sph_selftest_division(sph_ctx* ctx, uint64_t seed, uint64_t count, int mode, uint64_t* mismatches) {
    if (ctx == nullptr) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    return ctx->engine.selftest_division(seed, count, mode, mismatches);
}

int sph_launches_per_substep(const sph_ctx* ctx, uint32_t* launches) {
    if (ctx == nullptr || launches == nullptr) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    *launches = ctx->engine.launches_per_substep();
    return SPH_OK;
}

int sph_kernels_launched(const sph_ctx* ctx, uint64_t* kernels) {
    if (ctx == nullptr || kernels == nullptr) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    *kernels = ctx->engine.kernels_launched();
    return SPH_OK;
}

int sph_device_bytes(const sph_ctx* ctx, uint64_t* bytes) {
    if (ctx == nullptr || bytes == nullptr) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    *bytes = ctx->engine.device_bytes();
    return SPH_OK;
}

int sph_autotune(sph_ctx* ctx, float dt, uint32_t substeps_per_trial, sph_tuning* best, float* best_ms) {
    if (ctx == nullptr) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    return autotune(ctx->engine, dt, substeps_per_trial, best, best_ms);
}

// ---- batched tanks ----------------------------------------------------------

int sph_batch_create(const sph_params* params, const uint32_t* counts, uint32_t tanks, int device, sph_batch** out) {
    if (params == nullptr || counts == nullptr || out == nullptr || tanks == 0) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    *out = nullptr;
    std::vector<sph_params> p(params, params + tanks);
    std::vector<uint32_t> n(counts, counts + tanks);
    for (uint32_t c : n) {
        if (c == 0) {
            return SPH_ERR_INVALID_ARGUMENT;
        }
    }
    sph_batch* batch = new (std::nothrow) sph_batch();
    if (batch == nullptr) {
        return SPH_ERR_OUT_OF_MEMORY;
    }
    int status = batch->engine.init(device, p, n);
    if (status != SPH_OK) {
        delete batch;
        return status;
    }
    *out = batch;
    return SPH_OK;
}

int sph_batch_destroy(sph_batch* batch) {
    delete batch;
    return SPH_OK;
}

const char* sph_batch_last_error(const sph_batch* batch) { return batch == nullptr ? "" : batch->engine.last_error(); }

int sph_batch_tank_count(const sph_batch* batch, uint32_t* tanks) {
    if (batch == nullptr || tanks == nullptr) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    *tanks = batch->engine.tank_count();
    return SPH_OK;
}

int sph_batch_particle_count(const sph_batch* batch, uint32_t tank, uint32_t* count) {
    if (batch == nullptr || count == nullptr) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    if (tank == SPH_ALL_TANKS) {
        *count = batch->engine.total_count();
        return SPH_OK;
    }
    if (tank >= batch->engine.tank_count()) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    *count = batch->engine.count(tank);
    return SPH_OK;
}

int sph_batch_upload(sph_batch* batch, uint32_t tank, const float* positions, const float* velocities) {
    if (batch == nullptr || tank >= batch->engine.tank_count()) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    return batch->engine.upload(tank, positions, velocities, batch->engine.capacity(tank));
}

int sph_batch_download(sph_batch* batch, uint32_t tank, float* positions, float* velocities) {
    if (batch == nullptr || tank >= batch->engine.tank_count()) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    return batch->engine.download(tank, positions, velocities);
}

int sph_batch_emit(sph_batch* batch, uint32_t tank) {
    if (batch == nullptr || tank >= batch->engine.tank_count()) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    return batch->engine.emit(tank, batch->engine.capacity(tank));
}

int sph_batch_set_active(sph_batch* batch, const uint8_t* active) {
    if (batch == nullptr || active == nullptr) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    std::vector<uint8_t> a(active, active + batch->engine.tank_count());
    return batch->engine.set_active(a);
}

int sph_batch_run(sph_batch* batch, float dt, uint32_t substeps) {
    if (batch == nullptr) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    return batch->engine.run(dt, substeps);
}

int sph_batch_run_per_tank(sph_batch* batch, const float* dt, const uint32_t* substeps) {
    if (batch == nullptr || dt == nullptr || substeps == nullptr) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    uint32_t tanks = batch->engine.tank_count();
    return batch->engine.run_per_tank(std::vector<float>(dt, dt + tanks),
                                      std::vector<uint32_t>(substeps, substeps + tanks));
}

// FluidSolver::step for every tank: each tank splits the frame with its own
// fluidSubsteps (fluid_sph.cpp:311-321).
int sph_batch_step(sph_batch* batch, float delta_seconds) {
    if (batch == nullptr || std::isnan(delta_seconds)) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    if (delta_seconds <= 0.0F) {
        return SPH_OK;
    }
    uint32_t tanks = batch->engine.tank_count();
    std::vector<float> dt(tanks);
    std::vector<uint32_t> n(tanks);
    float frame_step = std::min(delta_seconds, SPH_MAX_FRAME_STEP);
    for (uint32_t t = 0; t < tanks; ++t) {
        n[t] = sph::fluid_substeps(batch->engine.params(t), delta_seconds);
        dt[t] = frame_step / static_cast<float>(n[t]);
    }
    return batch->engine.run_per_tank(dt, n);
}

int sph_batch_stats(sph_batch* batch, sph_stats* out) {
    if (batch == nullptr || out == nullptr) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    std::vector<sph_stats> all;
    int status = batch->engine.stats_all(all);
    if (status == SPH_OK) {
        std::copy(all.begin(), all.end(), out);
    }
    return status;
}

int sph_batch_synchronize(sph_batch* batch) {
    if (batch == nullptr) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    return batch->engine.synchronize();
}

int sph_batch_stream(sph_batch* batch, void** stream) {
    if (batch == nullptr || stream == nullptr) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    *stream = static_cast<void*>(batch->engine.stream());
    return SPH_OK;
}

int sph_batch_get_tuning(const sph_batch* batch, sph_tuning* out) {
    if (batch == nullptr || out == nullptr) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    sph::TuneChoice c;
    c.tuning = batch->engine.tuning();
    c.radix_bits = batch->engine.radix_bits();
    c.schedule = batch->engine.schedule_on();
    c.onesweep = batch->engine.onesweep_on();
    c.counting = batch->engine.counting_on();
    to_api(c, out);
    return SPH_OK;
}

int sph_batch_set_tuning(sph_batch* batch, const sph_tuning* tuning) {
    if (batch == nullptr || tuning == nullptr || tuning->schedule > 2 || tuning->sort > 2) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    sph::NeighbourTuning t = batch->engine.tuning();
    t.variant = tuning->neighbour_kernel;
    t.block = tuning->block_size;
    t.queue = tuning->queue_depth;
    int status = batch->engine.set_tuning(t);
    if (status == SPH_OK) {
        status = batch->engine.set_schedule(tuning->schedule);
    }
    if (status == SPH_OK) {
        status = batch->engine.set_onesweep(tuning->sort != 0);
    }
    if (status == SPH_OK) {
        status = batch->engine.set_counting(tuning->sort == 2);
    }
    if (status == SPH_OK) {
        status = batch->engine.set_radix_bits(tuning->radix_bits);
    }
    return status;
}

int sph_batch_autotune(sph_batch* batch, float dt, uint32_t substeps_per_trial, sph_tuning* best, float* best_ms) {
    if (batch == nullptr) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    return autotune(batch->engine, dt, substeps_per_trial, best, best_ms);
}

int sph_batch_profile_substeps(sph_batch* batch, float dt, uint32_t substeps, double* phase_ms) {
    if (batch == nullptr) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    return batch->engine.profile(dt, substeps, phase_ms);
}

int sph_batch_launches_per_substep(const sph_batch* batch, uint32_t* launches) {
    if (batch == nullptr || launches == nullptr) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    *launches = batch->engine.launches_per_substep();
    return SPH_OK;
}

int sph_batch_device_bytes(const sph_batch* batch, uint64_t* bytes) {
    if (batch == nullptr || bytes == nullptr) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    *bytes = batch->engine.device_bytes();
    return SPH_OK;
}

}  // extern "C"

// ---- learned coarse step --------------------------------------------------------

namespace {

int run_learned(sph::Engine& engine, float dt, uint32_t substeps, const sph_mlp* mlp) {
    sph::mlp::ModelView view{};
    const sph::mlp::ModelView* model = nullptr;
    if (mlp != nullptr) {
        if (!sph_mlp_model_view(mlp, &view)) {
            return SPH_ERR_INVALID_ARGUMENT;
        }
        model = &view;
    }
    return engine.run_learned(dt, substeps, model);
}

}  // namespace

extern "C" {

int sph_run_learned(sph_ctx* ctx, float dt, uint32_t substeps, const sph_mlp* mlp) {
    if (ctx == nullptr) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    return run_learned(ctx->engine, dt, substeps, mlp);
}

int sph_batch_run_learned(sph_batch* batch, float dt, uint32_t substeps, const sph_mlp* mlp) {
    if (batch == nullptr) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    return run_learned(batch->engine, dt, substeps, mlp);
}

int sph_batch_learned_features(sph_batch* batch, float dt, void* features) {
    if (batch == nullptr) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    return batch->engine.learned_features(dt, static_cast<float*>(features));
}

int sph_batch_learned_correction(sph_batch* batch, float dt, const sph_mlp* mlp, void* correction) {
    sph::mlp::ModelView view{};
    if (batch == nullptr || mlp == nullptr || !sph_mlp_model_view(mlp, &view)) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    return batch->engine.learned_correction(dt, view, static_cast<float4*>(correction));
}

int sph_batch_learned_check(sph_batch* batch) {
    if (batch == nullptr) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    return batch->engine.learned_error();
}

int sph_batch_snapshot(sph_batch* batch, uint32_t slot, int save) {
    if (batch == nullptr) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    return batch->engine.snapshot(save != 0, slot);
}

int sph_batch_restore_tanks(sph_batch* batch, uint32_t slot, const uint8_t* which) {
    if (batch == nullptr || which == nullptr) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    return batch->engine.restore_tanks(slot, std::vector<uint8_t>(which, which + batch->engine.tank_count()));
}

int sph_batch_device_state(sph_batch* batch, void** positions, void** velocities) {
    if (batch == nullptr) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    if (positions != nullptr) {
        *positions = batch->engine.positions();
    }
    if (velocities != nullptr) {
        *velocities = batch->engine.velocities();
    }
    return SPH_OK;
}

int sph_batch_copy_state(sph_batch* batch, void* positions, void* velocities) {
    if (batch == nullptr) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    return batch->engine.copy_state(static_cast<float4*>(positions), static_cast<float4*>(velocities));
}

int sph_batch_tank_offset(const sph_batch* batch, uint32_t tank, uint32_t* first) {
    if (batch == nullptr || first == nullptr || tank >= batch->engine.tank_count()) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    *first = batch->engine.particle_base(tank);
    return SPH_OK;
}

}  // extern "C"
