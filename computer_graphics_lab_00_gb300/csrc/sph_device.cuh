// sph_device.cuh — device-side types and helpers of the SPH step.
//
// Every float expression that feeds a result follows the reference's CPU
// solver operation by operation (src/physics/fluid_sph.cpp:24-309,
// src/physics/spatial_hash.h:12-20). The translation units that include this
// header are compiled with --fmad=false, so no a*b+c is fused and every
// operation rounds once, as the reference's x86-64 build does.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/sph_c.h"

namespace sph {

constexpr uint32_t kCellCapacity = 32;  // fluid_sph.h:23

// Per-tank constants. Everything that the reference recomputes per particle
// from FluidParams with the same float expression is computed once on the
// host with that expression (the kernel coefficients use the host's powf,
// exactly as the reference's std::pow(float, float)).
struct alignas(16) TankConst {
    float h;           // smoothing radius = cell size
    float h2;          // h * h
    float c_poly6;     // 315 / (64 * PI * pow(h, 9))
    float c_spiky;     // -45 / (PI * pow(h, 6))
    float c_visc;      // 45 / (PI * pow(h, 6))
    float mass;        // particle mass (gravity.w)
    float neg_mass;    // -mass
    float visc_mass;   // viscosity * mass
    float rest_density;
    float stiffness;
    float dt;          // substep length
    float max_speed;   // 0.4 * h / dt
    float r2_far;      // smallest r^2 whose rounded square root is >= h
    float r2_near;     // largest r^2 whose rounded square root is <= 1e-6
    float gravity[3];
    float restitution;
    float low[3];      // container_min + particle radius
    float rest_w;      // rest density written by emit
    float high[3];     // container_max - particle radius
    float spacing;
    uint32_t cell_mask;      // bucket count - 1
    uint32_t bucket_base;    // first global bucket of this tank
    uint32_t particle_base;  // first particle of this tank (id order)
    uint32_t particle_count;
    uint32_t lattice[3];
    uint32_t active;         // 0: the tank is frozen this substep
    float emitter_world[16];
    float radius;                      // particle radius (container_min.w)
    uint32_t collider_count;           // shape colliders of this tank (<= SPH_MAX_COLLIDERS)
    uint32_t field_count;              // force fields of this tank (<= SPH_MAX_FORCE_FIELDS)
    uint32_t curve_base;               // first cell bin of this tank (processing order of a batch)
    uint32_t curve_dims[3];            // the tank's cells a side from its low corner
    uint32_t pad_extra;
    const sph_collider* colliders;     // this tank's colliders in device memory
    const sph_force_field* fields;     // this tank's force fields in device memory
    const float4* field_accel;         // field accelerations of all particles (id order), if any tank has fields
};

struct StepCounters {
    unsigned long long candidates;
    unsigned long long in_range;
    unsigned int error_flags;
    unsigned int pad;
};

__device__ __forceinline__ int cell_coord(float p, float h) {
    // spatial_hash.h:12-14: int(floor(p / h)), IEEE division.
    return static_cast<int>(floorf(__fdiv_rn(p, h)));
}

__device__ __forceinline__ uint32_t spatial_hash(uint32_t cx, uint32_t cy, uint32_t cz, uint32_t mask) {
    // spatial_hash.h:16-20; the int -> uint casts are two's-complement.
    return ((cx * 73856093u) ^ (cy * 19349663u) ^ (cz * 83492791u)) & mask;
}

// glm::dot for vec3: (x*x' + y*y') + z*z', each operation rounded.
__device__ __forceinline__ float dot3(float x, float y, float z) {
    return __fadd_rn(__fadd_rn(__fmul_rn(x, x), __fmul_rn(y, y)), __fmul_rn(z, z));
}

// Correctly rounded x / y given r = RN(1/y): q = RN(x r) is within one ulp of
// x / y, the residual x - q y is exact in one FMA, and one more FMA rounds
// q + (x - q y) r to the correctly rounded quotient (Markstein's division
// theorem; P. Markstein, IBM J. Res. Dev. 34(1), 1990) as long as nothing
// overflows and the residual stays normal. Exhaustive GPU checks (every x
// from 2^-105 up to y, for y = r^2 at several r) found no difference; below
// about 2^-105 the residual underflows and about 0.3 % of quotients are one ulp
// off. Dividends here (mass times pressure sums, coordinate differences,
// mass times velocity differences) stay far above that in any physical state.
// A zero dividend yields +0 where
// IEEE division gives the dividend's signed zero; the sums it feeds start at
// +0 and so never change bits because of it.
constexpr float kDivByMinDividend = 0x1p-100f;  // checked exact at and above this dividend magnitude
__device__ __forceinline__ float div_by(float x, float y, float r) {
    float q = __fmul_rn(x, r);
    float e = __fmaf_rn(-q, y, x);
    return __fmaf_rn(e, r, q);
}

}  // namespace sph
