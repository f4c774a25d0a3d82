// sph_solver.hpp — header-only C++ wrapper over sph_c.h with the method
// names of the reference's physics::FluidSolver (src/physics/fluid_sph.h:101-127),
// so a FluidSimulator-style caller (src/gfx/fluid.cpp:396-399, :471-483) swaps
// the CPU solver for the GPU one by changing the type it holds.
//
//   physics::FluidSolver          gb::FluidSolverGpu
//   emit(params, count)           emit(params, count)
//   step(params, dt, jobs)        step(params, dt)         (no JobSystem: the GPU is the worker)
//   particles()                   particles()              (host copy, xyz position, w density)
//   previousParticles()           previousParticles()
//   keepRendered()                keepRendered()
//   particleCount()               particleCount()
//
// Errors surface as gb::SphError (a std::runtime_error carrying the status
// code); the C ABI underneath never aborts.
#pragma once

#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "sph_c.h"

namespace gb {

struct Float4 {
    float x, y, z, w;
};
static_assert(sizeof(Float4) == 16, "AoS float4 layout");

class SphError : public std::runtime_error {
public:
    SphError(int status, const std::string& what) : std::runtime_error(what), status_(status) {}
    int status() const { return status_; }

private:
    int status_;
};

inline void check(int status, const char* what, const sph_ctx* ctx = nullptr) {
    if (status != SPH_OK) {
        std::string text = std::string(what) + ": " + sph_status_string(status);
        if (ctx != nullptr && sph_last_error(ctx)[0] != '\0') {
            text += " (" + std::string(sph_last_error(ctx)) + ")";
        }
        throw SphError(status, text);
    }
}

class FluidSolverGpu {
public:
    FluidSolverGpu(const sph_params& params, uint32_t capacity, int device = 0) : params_(params) {
        check(sph_create(&params_, capacity, device, &ctx_), "sph_create");
    }
    ~FluidSolverGpu() { sph_destroy(ctx_); }
    FluidSolverGpu(const FluidSolverGpu&) = delete;
    FluidSolverGpu& operator=(const FluidSolverGpu&) = delete;

    void emit(const sph_params& params, uint32_t count) {
        use(params);
        check(sph_emit(ctx_, count), "sph_emit", ctx_);
    }

    void step(const sph_params& params, float deltaSeconds) {
        use(params);
        check(sph_step(ctx_, deltaSeconds), "sph_step", ctx_);
    }

    uint32_t particleCount() const {
        uint32_t n = 0;
        check(sph_particle_count(ctx_, &n), "sph_particle_count", ctx_);
        return n;
    }

    std::vector<Float4> particles() const {
        std::vector<Float4> out(particleCount());
        check(sph_download(ctx_, out.empty() ? nullptr : &out[0].x, nullptr), "sph_download", ctx_);
        return out;
    }

    // Velocities are private in the reference; offered here for tooling.
    std::vector<Float4> velocities() const {
        std::vector<Float4> out(particleCount());
        check(sph_download(ctx_, nullptr, out.empty() ? nullptr : &out[0].x), "sph_download", ctx_);
        return out;
    }

    std::vector<Float4> previousParticles() const {
        std::vector<Float4> out(particleCount());
        if (!out.empty()) {
            check(sph_download_previous(ctx_, &out[0].x), "sph_download_previous", ctx_);
        }
        return out;
    }

    void keepRendered() { check(sph_keep_rendered(ctx_), "sph_keep_rendered", ctx_); }

    // Loads a state (the reference fills it only through emit).
    void upload(const std::vector<Float4>& positions, const std::vector<Float4>* velocities = nullptr) {
        check(sph_upload(ctx_, positions.empty() ? nullptr : &positions[0].x,
                         velocities != nullptr && !velocities->empty() ? &(*velocities)[0].x : nullptr,
                         static_cast<uint32_t>(positions.size())),
              "sph_upload", ctx_);
    }

    // For a caller that keeps the state on the host: uploads it, runs
    // `substeps` substeps of `dt` and writes the result back in place, with
    // the copies overlapped where the passes allow (sph_step_host).
    void stepHost(std::vector<Float4>& positions, std::vector<Float4>& velocities, float dt, uint32_t substeps = 1) {
        if (velocities.size() != positions.size()) {
            throw std::invalid_argument("stepHost: positions and velocities differ in length");
        }
        float* p = positions.empty() ? nullptr : &positions[0].x;
        float* v = velocities.empty() ? nullptr : &velocities[0].x;
        check(sph_step_host(ctx_, p, v, static_cast<uint32_t>(positions.size()), dt, substeps, p, v),
              "sph_step_host", ctx_);
    }

    sph_ctx* handle() { return ctx_; }

private:
    void use(const sph_params& params) {
        if (std::memcmp(&params, &params_, sizeof(params)) != 0) {
            check(sph_set_params(ctx_, &params), "sph_set_params", ctx_);
            params_ = params;
        }
    }

    sph_params params_{};
    sph_ctx* ctx_ = nullptr;
};

}  // namespace gb
