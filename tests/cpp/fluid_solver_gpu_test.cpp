// The reference's fluid test blocks (tests/fluid_test.cpp:49-210), driven
// through the C++ wrapper gb::FluidSolverGpu on the GPU. Built and run by
// tests/test_cpp_wrapper.py; asserts stay on (-UNDEBUG).
#include <algorithm>
#include <cassert>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "sph_solver.hpp"

namespace {

// scene::Fluid defaults with the emitter at (0, 1, 0) (fluid_test.cpp:19-32).
sph_params paramsFor(uint32_t count, float half = 0.5F, float containerMinY = 0.0F) {
    sph_fluid_settings s{};
    for (int a = 0; a < 3; ++a) {
        s.emitter_half_extents[a] = half;
        s.container_min[a] = -1.0F;
        s.container_max[a] = 1.0F;
    }
    s.container_min[1] = containerMinY;
    s.container_max[1] = 2.0F;
    s.particle_radius = 0.025F;
    s.smoothing_radius = 0.1F;
    s.rest_density = 1000.0F;
    s.stiffness = 50.0F;
    s.viscosity = 0.5F;
    s.gravity[1] = -9.81F;
    float world[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 1, 0, 1};
    sph_params p{};
    gb::check(sph_derive_params(&s, world, count, 1024, &p), "sph_derive_params");
    return p;
}

bool insideContainer(const std::vector<gb::Float4>& particles, const sph_params& p) {
    for (const gb::Float4& q : particles) {
        const float v[3] = {q.x, q.y, q.z};
        for (int a = 0; a < 3; ++a) {
            if (v[a] < p.container_min[a] - 1e-3F || v[a] > p.container_max[a] + 1e-3F) {
                return false;
            }
        }
    }
    return true;
}

}  // namespace

int main() {
    // Emit lays a lattice inside the emitter box (fluid_test.cpp:53-75).
    {
        sph_params p = paramsFor(512, 0.4F);
        gb::FluidSolverGpu solver(p, 512);
        solver.emit(p, 512);
        assert(solver.particleCount() == 512);
        float half[3];
        for (int a = 0; a < 3; ++a) {
            half[a] = static_cast<float>(p.lattice[a] - 1U) * p.emitter_half_extents[3] * 0.5F;
        }
        std::vector<gb::Float4> particles = solver.particles();
        for (const gb::Float4& q : particles) {
            assert(std::abs(q.x) <= half[0] + 1e-4F);
            assert(std::abs(q.y - 1.0F) <= half[1] + 1e-4F);
        }
        assert(std::abs(particles[0].w - p.rest_density) < 1e-3F);
        std::vector<gb::Float4> previous = solver.previousParticles();
        assert(previous[0].x == particles[0].x && previous[0].y == particles[0].y && previous[0].z == particles[0].z);
    }
    // Particles stay in the container and settle (fluid_test.cpp:77-96).
    {
        sph_params p = paramsFor(512);
        gb::FluidSolverGpu solver(p, 512);
        solver.emit(p, 512);
        for (int frame = 0; frame < 60; ++frame) {
            solver.step(p, 1.0F / 60.0F);
        }
        std::vector<gb::Float4> particles = solver.particles();
        assert(insideContainer(particles, p));
        float highest = -1000.0F;
        for (const gb::Float4& q : particles) {
            highest = std::max(highest, q.y);
        }
        assert(highest < 0.6F);
    }
    // Same start, same result, bit for bit (fluid_test.cpp:130-150).
    {
        sph_params p = paramsFor(1024);
        gb::FluidSolverGpu first(p, 1024);
        gb::FluidSolverGpu second(p, 1024);
        first.emit(p, 1024);
        second.emit(p, 1024);
        for (int frame = 0; frame < 150; ++frame) {
            first.step(p, 1.0F / 60.0F);
            second.step(p, 1.0F / 60.0F);
        }
        std::vector<gb::Float4> a = first.particles();
        std::vector<gb::Float4> b = second.particles();
        for (size_t i = 0; i < a.size(); ++i) {
            assert(std::memcmp(&a[i], &b[i], sizeof(gb::Float4)) == 0);
        }
    }
    // stepHost (upload, substeps, download in one call, written back in
    // place) equals upload + substeps + particles()/velocities().
    {
        sph_params p = paramsFor(1024);
        gb::FluidSolverGpu device(p, 1024);
        gb::FluidSolverGpu host(p, 1024);
        device.emit(p, 1024);
        for (int frame = 0; frame < 10; ++frame) {
            device.step(p, 1.0F / 60.0F);
        }
        std::vector<gb::Float4> pos = device.particles();
        std::vector<gb::Float4> vel = device.velocities();
        for (int k = 0; k < 3; ++k) {
            gb::check(sph_substep(device.handle(), 1.0F / 600.0F), "sph_substep");
        }
        host.stepHost(pos, vel, 1.0F / 600.0F, 3);
        std::vector<gb::Float4> a = device.particles();
        std::vector<gb::Float4> b = device.velocities();
        for (size_t i = 0; i < a.size(); ++i) {
            assert(std::memcmp(&a[i], &pos[i], sizeof(gb::Float4)) == 0);
            assert(std::memcmp(&b[i], &vel[i], sizeof(gb::Float4)) == 0);
        }
    }
    // Parameter derivation (fluid_test.cpp:181-194).
    {
        sph_fluid_settings s{};
        for (int a = 0; a < 3; ++a) {
            s.emitter_half_extents[a] = 0.5F;
        }
        s.particle_radius = 0.05F;
        s.rest_density = 1000.0F;
        s.smoothing_radius = 0.01F;
        float world[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 1, 0, 1};
        sph_params p{};
        gb::check(sph_derive_params(&s, world, 100, 1024, &p), "sph_derive_params");
        assert(std::abs(p.emitter_half_extents[3] - 0.1F) < 1e-6F);
        assert(std::abs(p.gravity[3] - 1000.0F * 0.001F) < 1e-4F);
        assert(p.smoothing_radius >= p.emitter_half_extents[3]);
        assert(p.lattice[3] == 1024);
    }
    // Substeps lie in [1, 8] (fluid_test.cpp:196-207).
    {
        sph_params p = paramsFor(100);
        uint32_t n = 0;
        gb::check(sph_fluid_substeps(&p, 0.0F, &n), "substeps");
        assert(n == 1);
        p.stiffness = 100000.0F;
        gb::check(sph_fluid_substeps(&p, 1.0F / 60.0F, &n), "substeps");
        assert(n == 8);
        p.stiffness = 1.0F;
        p.smoothing_radius = 10.0F;
        gb::check(sph_fluid_substeps(&p, 1.0F / 60.0F, &n), "substeps");
        assert(n == 1);
        gb::check(sph_fluid_substeps(&p, 100.0F, &n), "substeps");
        assert(n <= 8);
    }
    // Errors are exceptions carrying the status, not aborts.
    {
        sph_params p = paramsFor(16);
        p.lattice[3] = 1000;
        bool threw = false;
        try {
            gb::FluidSolverGpu bad(p, 16);
        } catch (const gb::SphError& e) {
            threw = e.status() == SPH_ERR_INVALID_ARGUMENT;
        }
        assert(threw);
    }
    std::printf("gb::FluidSolverGpu: reference fluid test blocks passed\n");
    return 0;
}
