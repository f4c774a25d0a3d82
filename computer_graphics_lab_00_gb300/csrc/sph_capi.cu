// sph_capi.cu — the extern "C" entry points of include/sph_c.h.
//
// Each entry point checks its arguments, forwards to the Engine and returns
// a status code; none aborts. The context is the GPU counterpart of one
// physics::FluidSolver (src/physics/fluid_sph.h:101-127).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>

#include "../../include/sph_c.h"
#include "sph_engine.h"

struct sph_ctx {
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
    out->schedule = ctx->engine.schedule_on() ? 1u : 0u;
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
    if (tuning->schedule > 1) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    int status = ctx->engine.set_tuning(t);
    if (status != SPH_OK) {
        return status;
    }
    status = ctx->engine.set_schedule(tuning->schedule != 0);
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

int sph_device_bytes(const sph_ctx* ctx, uint64_t* bytes) {
    if (ctx == nullptr || bytes == nullptr) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    *bytes = ctx->engine.device_bytes();
    return SPH_OK;
}

}  // extern "C"
