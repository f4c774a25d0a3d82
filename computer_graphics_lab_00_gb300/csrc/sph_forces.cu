// sph_forces.cu — density/pressure and force/integrate passes, emit and
// statistics.
//
// One thread per particle in cell order: particle p of the sorted arrays
// reads its own row, walks the 27 neighbour buckets in the reference's
// (dz, dy, dx) order and, inside a bucket, the first min(count, 32) entries in
// id order — the summation order of src/physics/fluid_sph.cpp:205-216 and
// :234-258, so the sums round exactly as the reference's do. Because the
// arrays are cell-ordered, the lanes of a warp that share a cell read the same
// neighbour rows, and each neighbour row is one aligned 16-byte load.
//
// Compiled with --fmad=false; the explicit __f*_rn intrinsics state the
// rounding of each operation.
#include "sph_kernels.h"
#include "sph_mlp.cuh"

#include <algorithm>
#include <mutex>
#include <type_traits>

namespace sph {

namespace {

// std::max(a, b) returns b only when a < b.
__device__ __forceinline__ float max_like_std(float a, float b) { return a < b ? b : a; }

__device__ __forceinline__ void finish_particle(const TankConst* t, const float4& self, float density, float vx,
                                                float vy, float vz, float pressure, float fx, float fy, float fz,
                                                uint32_t i, float4* __restrict__ pos_out,
                                                float4* __restrict__ vel_out,
                                                float4 learned = {0.0f, 0.0f, 0.0f, 0.0f});

template <bool kCount>
__global__ void __launch_bounds__(128) density_kernel(const float4* __restrict__ spos, float4* __restrict__ svel,
                                                      float4* __restrict__ spos2, const uint2* __restrict__ bucket,
                                                      const TankConst* __restrict__ tanks,
                                                      const uint16_t* __restrict__ stank, uint32_t n, const uint32_t* __restrict__ order,
                                                      StepCounters* __restrict__ counters) {
    uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (order != nullptr && p < n) {
        p = order[p];
    }
    if (p >= n) {
        return;
    }
    const TankConst* t = tanks + (stank != nullptr ? stank[p] : 0);
    const float h = __ldg(&t->h);
    const float h2 = __ldg(&t->h2);
    const float c6 = __ldg(&t->c_poly6);
    const float mass = __ldg(&t->mass);
    const uint32_t mask = __ldg(&t->cell_mask);
    const uint32_t base = __ldg(&t->bucket_base);
    const float4 self = spos[p];
    const uint32_t cx = static_cast<uint32_t>(cell_coord(self.x, h));
    const uint32_t cy = static_cast<uint32_t>(cell_coord(self.y, h));
    const uint32_t cz = static_cast<uint32_t>(cell_coord(self.z, h));
    float density = 0.0f;
    uint32_t candidates = 0;
    uint32_t in_range = 0;
    for (int dz = -1; dz <= 1; ++dz) {
        for (int dy = -1; dy <= 1; ++dy) {
            for (int dx = -1; dx <= 1; ++dx) {
                uint32_t b = base + spatial_hash(cx + static_cast<uint32_t>(dx), cy + static_cast<uint32_t>(dy),
                                                 cz + static_cast<uint32_t>(dz), mask);
                uint2 range = __ldg(&bucket[b]);
                uint32_t count = min(range.y - range.x, kCellCapacity);
                if (kCount) {
                    candidates += count;
                }
                for (uint32_t q = range.x; q < range.x + count; ++q) {
                    float4 other = __ldg(&spos[q]);
                    float ex = __fsub_rn(self.x, other.x);
                    float ey = __fsub_rn(self.y, other.y);
                    float ez = __fsub_rn(self.z, other.z);
                    float r2 = dot3(ex, ey, ez);
                    if (r2 < h2) {
                        // poly6 (fluid_sph.cpp:24-31) times mass, added in order.
                        float d = __fsub_rn(h2, r2);
                        float w = __fmul_rn(__fmul_rn(__fmul_rn(c6, d), d), d);
                        density = __fadd_rn(density, __fmul_rn(mass, w));
                        if (kCount) {
                            ++in_range;
                        }
                    }
                }
            }
        }
    }
    density = max_like_std(density, 1e-6f);
    float pressure =
        max_like_std(__fmul_rn(__ldg(&t->stiffness), __fsub_rn(density, __ldg(&t->rest_density))), 0.0f);
    spos2[p] = make_float4(self.x, self.y, self.z, density);
    reinterpret_cast<float*>(svel)[4 * static_cast<size_t>(p) + 3] = pressure;
    if (kCount) {
        unsigned long long c = candidates;
        unsigned long long r = in_range;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            c += __shfl_down_sync(0xFFFFFFFFu, c, o);
            r += __shfl_down_sync(0xFFFFFFFFu, r, o);
        }
        if ((threadIdx.x & 31) == 0) {
            atomicAdd(&counters->candidates, c);
            atomicAdd(&counters->in_range, r);
        }
    }
}

__global__ void __launch_bounds__(128) integrate_kernel(const float4* __restrict__ spos2,
                                                        const float4* __restrict__ svel,
                                                        const uint32_t* __restrict__ sorted_ids,
                                                        const uint2* __restrict__ bucket,
                                                        const TankConst* __restrict__ tanks,
                                                        const uint16_t* __restrict__ stank, uint32_t n, const uint32_t* __restrict__ order,
                                                        float4* __restrict__ pos_out, float4* __restrict__ vel_out) {
    uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (order != nullptr && p < n) {
        p = order[p];
    }
    if (p >= n) {
        return;
    }
    const TankConst* t = tanks + (stank != nullptr ? stank[p] : 0);
    if (__ldg(&t->active) == 0) {
        return;
    }
    const float h = __ldg(&t->h);
    const float c_spiky = __ldg(&t->c_spiky);
    const float c_visc = __ldg(&t->c_visc);
    const float neg_mass = __ldg(&t->neg_mass);
    const float visc_mass = __ldg(&t->visc_mass);
    const uint32_t mask = __ldg(&t->cell_mask);
    const uint32_t base = __ldg(&t->bucket_base);

    const float4 self = spos2[p];
    const float density = max_like_std(self.w, 1e-6f);
    const float4 self_vel = svel[p];
    float vx = self_vel.x;
    float vy = self_vel.y;
    float vz = self_vel.z;
    const float pressure = self_vel.w;
    const uint32_t cx = static_cast<uint32_t>(cell_coord(self.x, h));
    const uint32_t cy = static_cast<uint32_t>(cell_coord(self.y, h));
    const uint32_t cz = static_cast<uint32_t>(cell_coord(self.z, h));

    float fx = 0.0f;
    float fy = 0.0f;
    float fz = 0.0f;
    for (int dz = -1; dz <= 1; ++dz) {
        for (int dy = -1; dy <= 1; ++dy) {
            for (int dx = -1; dx <= 1; ++dx) {
                uint32_t b = base + spatial_hash(cx + static_cast<uint32_t>(dx), cy + static_cast<uint32_t>(dy),
                                                 cz + static_cast<uint32_t>(dz), mask);
                uint2 range = __ldg(&bucket[b]);
                uint32_t count = min(range.y - range.x, kCellCapacity);
                for (uint32_t q = range.x; q < range.x + count; ++q) {
                    if (q == p) {
                        continue;
                    }
                    float4 other = __ldg(&spos2[q]);
                    float ex = __fsub_rn(self.x, other.x);
                    float ey = __fsub_rn(self.y, other.y);
                    float ez = __fsub_rn(self.z, other.z);
                    float distance = __fsqrt_rn(dot3(ex, ey, ez));
                    if (distance >= h || distance <= 1e-6f) {
                        continue;
                    }
                    float other_density = max_like_std(other.w, 1e-6f);
                    float4 ov = __ldg(&svel[q]);
                    // -m (p_i + p_j) / (2 rho_j) * spikyGradient (fluid_sph.cpp:251-252, :33-39).
                    float ps = __fdiv_rn(__fmul_rn(neg_mass, __fadd_rn(pressure, ov.w)),
                                         __fmul_rn(2.0f, other_density));
                    float d = __fsub_rn(h, distance);
                    float gs = __fmul_rn(__fmul_rn(c_spiky, d), d);
                    fx = __fadd_rn(fx, __fmul_rn(ps, __fmul_rn(gs, __fdiv_rn(ex, distance))));
                    fy = __fadd_rn(fy, __fmul_rn(ps, __fmul_rn(gs, __fdiv_rn(ey, distance))));
                    fz = __fadd_rn(fz, __fmul_rn(ps, __fmul_rn(gs, __fdiv_rn(ez, distance))));
                    // mu m (v_j - v_i) / rho_j * viscosityLaplacian (fluid_sph.cpp:253-254, :41-46).
                    float lap = __fmul_rn(c_visc, d);
                    fx = __fadd_rn(fx, __fmul_rn(__fdiv_rn(__fmul_rn(visc_mass, __fsub_rn(ov.x, vx)), other_density), lap));
                    fy = __fadd_rn(fy, __fmul_rn(__fdiv_rn(__fmul_rn(visc_mass, __fsub_rn(ov.y, vy)), other_density), lap));
                    fz = __fadd_rn(fz, __fmul_rn(__fdiv_rn(__fmul_rn(visc_mass, __fsub_rn(ov.z, vz)), other_density), lap));
                }
            }
        }
    }

    finish_particle(t, self, density, vx, vy, vz, pressure, fx, fy, fz, sorted_ids[p], pos_out, vel_out);
}

// The 27 neighbour buckets of a cell, in the reference's (dz, dy, dx) order
// (fluid_sph.cpp:205-207): walk index b = 9 (dz + 1) + 3 (dy + 1) + (dx + 1).
__device__ __forceinline__ uint2 neighbour_range(const uint2* __restrict__ bucket, uint32_t cx, uint32_t cy,
                                                 uint32_t cz, uint32_t b, uint32_t mask, uint32_t base) {
    uint32_t dz = b / 9u;
    uint32_t dy = (b / 3u) % 3u;
    uint32_t dx = b % 3u;
    uint32_t key = base + spatial_hash(cx + dx - 1u, cy + dy - 1u, cz + dz - 1u, mask);
    uint2 range = __ldg(&bucket[key]);
    return make_uint2(range.x, range.x + min(range.y - range.x, kCellCapacity));
}

// Density with one flat loop over the concatenated 27-bucket candidate
// stream, so lanes whose cells have different bucket sizes stay converged
// for as long as their streams last.
template <bool kCount>
__global__ void density_flat_kernel(const float4* __restrict__ spos, float4* __restrict__ svel,
                                    float4* __restrict__ spos2, const uint2* __restrict__ bucket,
                                    const TankConst* __restrict__ tanks, const uint16_t* __restrict__ stank,
                                    uint32_t n, const uint32_t* __restrict__ order, StepCounters* __restrict__ counters) {
    uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (order != nullptr && p < n) {
        p = order[p];
    }
    bool valid = p < n;
    const TankConst* t = tanks + (valid && stank != nullptr ? stank[p] : 0);
    const float h = __ldg(&t->h);
    const float h2 = __ldg(&t->h2);
    const float c6 = __ldg(&t->c_poly6);
    const float mass = __ldg(&t->mass);
    const uint32_t mask = __ldg(&t->cell_mask);
    const uint32_t base = __ldg(&t->bucket_base);
    const float4 self = valid ? spos[p] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    const uint32_t cx = static_cast<uint32_t>(cell_coord(self.x, h));
    const uint32_t cy = static_cast<uint32_t>(cell_coord(self.y, h));
    const uint32_t cz = static_cast<uint32_t>(cell_coord(self.z, h));
    float density = 0.0f;
    uint32_t candidates = 0;
    uint32_t in_range = 0;
    uint32_t b = valid ? 0u : 27u;
    uint32_t cur = 0;
    uint32_t end = 0;
    for (;;) {
        while (cur == end && b < 27u) {
            uint2 r = neighbour_range(bucket, cx, cy, cz, b, mask, base);
            cur = r.x;
            end = r.y;
            ++b;
            if (kCount) {
                candidates += end - cur;
            }
        }
        if (cur == end) {
            break;
        }
        float4 other = __ldg(&spos[cur]);
        ++cur;
        float ex = __fsub_rn(self.x, other.x);
        float ey = __fsub_rn(self.y, other.y);
        float ez = __fsub_rn(self.z, other.z);
        float r2 = dot3(ex, ey, ez);
        if (r2 < h2) {
            // poly6 (fluid_sph.cpp:24-31) times mass, added in candidate order.
            float d = __fsub_rn(h2, r2);
            float w = __fmul_rn(__fmul_rn(__fmul_rn(c6, d), d), d);
            density = __fadd_rn(density, __fmul_rn(mass, w));
            if (kCount) {
                ++in_range;
            }
        }
    }
    if (kCount) {
        unsigned long long c = candidates;
        unsigned long long r = in_range;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            c += __shfl_down_sync(0xFFFFFFFFu, c, o);
            r += __shfl_down_sync(0xFFFFFFFFu, r, o);
        }
        if ((threadIdx.x & 31) == 0) {
            atomicAdd(&counters->candidates, c);
            atomicAdd(&counters->in_range, r);
        }
    }
    if (!valid) {
        return;
    }
    density = max_like_std(density, 1e-6f);
    float pressure =
        max_like_std(__fmul_rn(__ldg(&t->stiffness), __fsub_rn(density, __ldg(&t->rest_density))), 0.0f);
    spos2[p] = make_float4(self.x, self.y, self.z, density);
    reinterpret_cast<float*>(svel)[4 * static_cast<size_t>(p) + 3] = pressure;
}

struct PairConst {
    float h, c_spiky, c_visc, neg_mass, visc_mass;
};

// Pressure and viscosity force of one in-range pair, added to f in the
// reference's order (fluid_sph.cpp:244-254).
__device__ __forceinline__ void add_pair_force(const PairConst& k, const float4& self, float vx, float vy, float vz,
                                               float pressure, const float4& other, const float4& ov, float& fx,
                                               float& fy, float& fz) {
    float ex = __fsub_rn(self.x, other.x);
    float ey = __fsub_rn(self.y, other.y);
    float ez = __fsub_rn(self.z, other.z);
    float distance = __fsqrt_rn(dot3(ex, ey, ez));
    float other_density = max_like_std(other.w, 1e-6f);
    float ps = __fdiv_rn(__fmul_rn(k.neg_mass, __fadd_rn(pressure, ov.w)), __fmul_rn(2.0f, other_density));
    float d = __fsub_rn(k.h, distance);
    float gs = __fmul_rn(__fmul_rn(k.c_spiky, d), d);
    fx = __fadd_rn(fx, __fmul_rn(ps, __fmul_rn(gs, __fdiv_rn(ex, distance))));
    fy = __fadd_rn(fy, __fmul_rn(ps, __fmul_rn(gs, __fdiv_rn(ey, distance))));
    fz = __fadd_rn(fz, __fmul_rn(ps, __fmul_rn(gs, __fdiv_rn(ez, distance))));
    float lap = __fmul_rn(k.c_visc, d);
    fx = __fadd_rn(fx, __fmul_rn(__fdiv_rn(__fmul_rn(k.visc_mass, __fsub_rn(ov.x, vx)), other_density), lap));
    fy = __fadd_rn(fy, __fmul_rn(__fdiv_rn(__fmul_rn(k.visc_mass, __fsub_rn(ov.y, vy)), other_density), lap));
    fz = __fadd_rn(fz, __fmul_rn(__fdiv_rn(__fmul_rn(k.visc_mass, __fsub_rn(ov.z, vz)), other_density), lap));
}

// ---- force fields and shape colliders -------------------------------------------
//
// Both follow the reference operation by operation: force_field.h:31-70 and
// collider_shapes.h:27-134 with fluid_sph.cpp:48-53 and :287-300. They sit
// in kernels of their own, launched only when some tank has fields or
// colliders: `fields_kernel` sums the field accelerations at the substep's
// start positions before integrate reads them, and `colliders_kernel`
// pushes particles out after integrate has applied the walls, which is where
// the reference's collider loop sits. The neighbour kernels carry no trace of
// either beyond one uniform branch.

// std::clamp(v, lo, hi) and std::min / std::max.
__device__ __forceinline__ float clamp_like_std(float v, float lo, float hi) { return v < lo ? lo : (hi < v ? hi : v); }
__device__ __forceinline__ float min_like_std(float a, float b) { return b < a ? b : a; }

// std::pow(float, float) of the reference, used for the field falloff. The
// power is evaluated in double and rounded once to float: the correctly
// rounded powf (except where the double result falls within its own error of
// a float rounding boundary). The host's glibc powf is not correctly rounded:
// on about 0.1 % of arguments in (0, 1) it returns the neighbouring float, so
// a falloff other than 1 agrees with the reference to 1 ulp in the weight;
// a falloff of 1 or a radius of 0 (no power) is bit-exact.
//
// The two common falloffs skip the double-precision power, whose cost
// dominates a field pass on a part with a low FP64 rate: x^1 is x itself
// (the double result lies within a few double ulps of the float x and rounds
// back to it) and x^0 is 1 for every x, so both shortcuts return the same
// bits as the general path.
__device__ __forceinline__ float pow_float(float x, float y) {
    if (y == 1.0f) {
        return x;
    }
    if (y == 0.0f) {
        return 1.0f;
    }
    return __double2float_rn(pow(static_cast<double>(x), static_cast<double>(y)));
}

// forceFieldsAcceleration (force_field.h:62-70): +0 plus every field in order.
__device__ __forceinline__ float3 fields_acceleration(const sph_force_field* __restrict__ fields, uint32_t count,
                                                   float x, float y, float z) {
    float tx = 0.0f, ty = 0.0f, tz = 0.0f;
    for (uint32_t i = 0; i < count; ++i) {
        const sph_force_field& f = fields[i];
        float ox = __fsub_rn(x, f.position_radius[0]);
        float oy = __fsub_rn(y, f.position_radius[1]);
        float oz = __fsub_rn(z, f.position_radius[2]);
        float distance = __fsqrt_rn(dot3(ox, oy, oz));
        float weight = 1.0f;
        float radius = f.position_radius[3];
        if (radius > 0.0f) {
            float t = clamp_like_std(__fsub_rn(1.0f, __fdiv_rn(distance, radius)), 0.0f, 1.0f);
            weight = t <= 0.0f ? 0.0f : pow_float(t, f.falloff);
        }
        float ax = 0.0f, ay = 0.0f, az = 0.0f;
        if (!(weight <= 0.0f)) {
            float s = __fmul_rn(f.axis_strength[3], weight);
            float kx = f.axis_strength[0], ky = f.axis_strength[1], kz = f.axis_strength[2];
            if (f.type == 0) {
                ax = __fmul_rn(kx, s);
                ay = __fmul_rn(ky, s);
                az = __fmul_rn(kz, s);
            } else if (f.type == 1) {
                float along = __fadd_rn(__fadd_rn(__fmul_rn(ox, kx), __fmul_rn(oy, ky)), __fmul_rn(oz, kz));
                float rx = __fsub_rn(ox, __fmul_rn(kx, along));
                float ry = __fsub_rn(oy, __fmul_rn(ky, along));
                float rz = __fsub_rn(oz, __fmul_rn(kz, along));
                float r = __fsqrt_rn(dot3(rx, ry, rz));
                if (!(r < 1.0e-4f)) {
                    float ux = __fdiv_rn(rx, r), uy = __fdiv_rn(ry, r), uz = __fdiv_rn(rz, r);
                    // glm::cross(axis, u).
                    ax = __fmul_rn(__fsub_rn(__fmul_rn(ky, uz), __fmul_rn(uy, kz)), s);
                    ay = __fmul_rn(__fsub_rn(__fmul_rn(kz, ux), __fmul_rn(uz, kx)), s);
                    az = __fmul_rn(__fsub_rn(__fmul_rn(kx, uy), __fmul_rn(ux, ky)), s);
                }
            } else if (f.type == 2) {
                if (!(distance < 1.0e-4f)) {
                    ax = __fmul_rn(__fdiv_rn(-ox, distance), s);
                    ay = __fmul_rn(__fdiv_rn(-oy, distance), s);
                    az = __fmul_rn(__fdiv_rn(-oz, distance), s);
                }
            }
        }
        tx = __fadd_rn(tx, ax);
        ty = __fadd_rn(ty, ay);
        tz = __fadd_rn(tz, az);
    }
    return make_float3(tx, ty, tz);
}

struct SurfacePoint {
    float p[3];
    float n[3];
    float d;
};

// closestOnSphereLocal (collider_shapes.h:33-41).
__device__ __forceinline__ SurfacePoint closest_on_sphere(float radius, float x, float y, float z) {
    SurfacePoint r;
    float d = __fsqrt_rn(dot3(x, y, z));
    if (d > 1.0e-6f) {
        r.n[0] = __fdiv_rn(x, d);
        r.n[1] = __fdiv_rn(y, d);
        r.n[2] = __fdiv_rn(z, d);
    } else {
        r.n[0] = 0.0f;
        r.n[1] = 1.0f;
        r.n[2] = 0.0f;
    }
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        r.p[a] = __fmul_rn(r.n[a], radius);
    }
    r.d = __fsub_rn(d, radius);
    return r;
}

// closestOnBoxLocal (collider_shapes.h:44-66); glm::clamp = min(max(v, lo), hi).
__device__ __forceinline__ SurfacePoint closest_on_box(const float* e, const float* p) {
    SurfacePoint r;
    float c[3], dl[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        c[a] = min_like_std(max_like_std(p[a], -e[a]), e[a]);
        dl[a] = __fsub_rn(p[a], c[a]);
    }
    float dist_sq = dot3(dl[0], dl[1], dl[2]);
    if (dist_sq > 1.0e-10f) {
        float dist = __fsqrt_rn(dist_sq);
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            r.n[a] = __fdiv_rn(dl[a], dist);
            r.p[a] = c[a];
        }
        r.d = dist;
        return r;
    }
    float gap[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        gap[a] = __fsub_rn(e[a], fabsf(p[a]));
    }
    int axis = gap[0] < gap[1] ? (gap[0] < gap[2] ? 0 : 2) : (gap[1] < gap[2] ? 1 : 2);
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        r.n[a] = 0.0f;
        r.p[a] = p[a];
    }
    float sign = p[axis] >= 0.0f ? 1.0f : -1.0f;
    r.n[axis] = sign;
    r.p[axis] = __fmul_rn(sign, e[axis]);
    r.d = -gap[axis];
    return r;
}

// closestOnCylinderLocal (collider_shapes.h:85-115).
__device__ __forceinline__ SurfacePoint closest_on_cylinder(float radius, float half_height, const float* p) {
    SurfacePoint r;
    float d = __fsqrt_rn(dot3(p[0], 0.0f, p[2]));
    float dir[3];
    if (d > 1.0e-6f) {
        dir[0] = __fdiv_rn(p[0], d);
        dir[1] = __fdiv_rn(0.0f, d);
        dir[2] = __fdiv_rn(p[2], d);
    } else {
        dir[0] = 1.0f;
        dir[1] = 0.0f;
        dir[2] = 0.0f;
    }
    bool inside = fabsf(p[1]) <= half_height && d <= radius;
    if (inside) {
        float gap_y = __fsub_rn(half_height, fabsf(p[1]));
        float gap_r = __fsub_rn(radius, d);
        if (gap_y < gap_r) {
            float side = p[1] >= 0.0f ? 1.0f : -1.0f;
            r.n[0] = 0.0f;
            r.n[1] = side;
            r.n[2] = 0.0f;
            r.p[0] = p[0];
            r.p[1] = __fmul_rn(side, half_height);
            r.p[2] = p[2];
            r.d = -gap_y;
        } else {
            const float add[3] = {0.0f, p[1], 0.0f};
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                r.n[a] = dir[a];
                r.p[a] = __fadd_rn(__fmul_rn(dir[a], radius), add[a]);
            }
            r.d = -gap_r;
        }
        return r;
    }
    float reach = min_like_std(d, radius);
    float c[3] = {__fmul_rn(dir[0], reach), __fmul_rn(dir[1], reach), __fmul_rn(dir[2], reach)};
    c[1] = clamp_like_std(p[1], -half_height, half_height);
    float dl[3] = {__fsub_rn(p[0], c[0]), __fsub_rn(p[1], c[1]), __fsub_rn(p[2], c[2])};
    float dist = __fsqrt_rn(dot3(dl[0], dl[1], dl[2]));
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        r.p[a] = c[a];
    }
    if (dist > 1.0e-6f) {
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            r.n[a] = __fdiv_rn(dl[a], dist);
        }
    } else {
        r.n[0] = 0.0f;
        r.n[1] = 1.0f;
        r.n[2] = 0.0f;
    }
    r.d = dist;
    return r;
}

// closestOnColliderLocal (collider_shapes.h:118-134).
__device__ __forceinline__ SurfacePoint closest_on_collider(const sph_collider& c, const float* p) {
    const float radius = c.data0[3];
    switch (c.type) {
    case 0:
        return closest_on_sphere(radius, p[0], p[1], p[2]);
    case 1:
        return closest_on_box(c.data0, p);
    case 2: {
        SurfacePoint r;  // closestOnPlaneLocal (collider_shapes.h:68-74)
        r.n[0] = 0.0f;
        r.n[1] = 1.0f;
        r.n[2] = 0.0f;
        r.p[0] = p[0];
        r.p[1] = 0.0f;
        r.p[2] = p[2];
        r.d = p[1];
        return r;
    }
    case 3:
        return closest_on_cylinder(radius, c.data0[1], p);
    case 4: {
        // closestOnCapsuleLocal (collider_shapes.h:77-82).
        float hh = c.data0[1];
        float seg = clamp_like_std(p[1], -hh, hh);
        SurfacePoint r = closest_on_sphere(radius, __fsub_rn(p[0], 0.0f), __fsub_rn(p[1], seg), __fsub_rn(p[2], 0.0f));
        r.p[0] = __fadd_rn(r.p[0], 0.0f);
        r.p[1] = __fadd_rn(r.p[1], seg);
        r.p[2] = __fadd_rn(r.p[2], 0.0f);
        return r;
    }
    default:
        return closest_on_sphere(0.0f, p[0], p[1], p[2]);
    }
}

// glm mat4 * vec4(v, w) for column-major m: (c0 x + c1 y) + (c2 z + c3 w).
__device__ __forceinline__ float mat4_row(const float* m, int r, const float* v, float w) {
    return __fadd_rn(__fadd_rn(__fmul_rn(m[r], v[0]), __fmul_rn(m[4 + r], v[1])),
                     __fadd_rn(__fmul_rn(m[8 + r], v[2]), __fmul_rn(m[12 + r], w)));
}

// One-way shape colliders (fluid_sph.cpp:287-300), in order, each seeing the
// position the previous one left; bounce is fluid_sph.cpp:48-53.
__device__ __forceinline__ void apply_colliders(const sph_collider* __restrict__ colliders, uint32_t count,
                                                float particle_radius, float restitution, float* pp, float* vv) {
    for (uint32_t c = 0; c < count; ++c) {
        const sph_collider& col = colliders[c];
        float local[3];
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            local[r] = mat4_row(col.inverse_world, r, pp, 1.0f);
        }
        SurfacePoint s = closest_on_collider(col, local);
        if (s.d < particle_radius) {
            // glm::normalize(mat3(world) * n) = v * (1 / sqrt(dot(v, v))).
            float nv[3];
#pragma unroll
            for (int r = 0; r < 3; ++r) {
                nv[r] = __fadd_rn(__fadd_rn(__fmul_rn(col.world[r], s.n[0]), __fmul_rn(col.world[4 + r], s.n[1])),
                                  __fmul_rn(col.world[8 + r], s.n[2]));
            }
            float inv = __fdiv_rn(1.0f, __fsqrt_rn(dot3(nv[0], nv[1], nv[2])));
#pragma unroll
            for (int r = 0; r < 3; ++r) {
                nv[r] = __fmul_rn(nv[r], inv);
            }
            float moved[3];
#pragma unroll
            for (int r = 0; r < 3; ++r) {
                moved[r] = __fadd_rn(mat4_row(col.world, r, s.p, 1.0f), __fmul_rn(nv[r], particle_radius));
            }
#pragma unroll
            for (int r = 0; r < 3; ++r) {
                pp[r] = moved[r];
            }
            float along = __fadd_rn(__fadd_rn(__fmul_rn(vv[0], nv[0]), __fmul_rn(vv[1], nv[1])), __fmul_rn(vv[2], nv[2]));
            if (along < 0.0f) {
                float k = __fmul_rn(__fadd_rn(1.0f, restitution), along);
#pragma unroll
                for (int r = 0; r < 3; ++r) {
                    vv[r] = __fsub_rn(vv[r], __fmul_rn(k, nv[r]));
                }
            }
        }
    }
}

// forceFieldsAcceleration at each particle's position (id order), for the
// tanks that have fields.
__global__ void fields_kernel(const float4* __restrict__ pos, const uint16_t* __restrict__ tank_of,
                              const TankConst* __restrict__ tanks, uint32_t n, float4* __restrict__ out) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) {
        return;
    }
    const TankConst* t = tanks + (tank_of != nullptr ? tank_of[i] : 0);
    uint32_t count = t->field_count;
    if (count == 0 || t->active == 0) {
        return;
    }
    float4 p = pos[i];
    float3 a = fields_acceleration(t->fields, count, p.x, p.y, p.z);
    out[i] = make_float4(a.x, a.y, a.z, 0.0f);
}

// The collider loop of fluid_sph.cpp:287-300 on the integrated state (id
// order), for the tanks that have colliders.
__global__ void colliders_kernel(float4* __restrict__ pos, float4* __restrict__ vel,
                                 const uint16_t* __restrict__ tank_of, const TankConst* __restrict__ tanks,
                                 uint32_t n) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) {
        return;
    }
    const TankConst* t = tanks + (tank_of != nullptr ? tank_of[i] : 0);
    uint32_t count = t->collider_count;
    if (count == 0 || t->active == 0) {
        return;
    }
    float4 p = pos[i];
    float4 v = vel[i];
    float pp[3] = {p.x, p.y, p.z};
    float vv[3] = {v.x, v.y, v.z};
    apply_colliders(t->colliders, count, t->radius, t->restitution, pp, vv);
    pos[i] = make_float4(pp[0], pp[1], pp[2], p.w);
    vel[i] = make_float4(vv[0], vv[1], vv[2], v.w);
}

// Semi-implicit Euler, speed clamp and walls (fluid_sph.cpp:260-285), then
// the id-order write.
__device__ __forceinline__ void finish_particle(const TankConst* t, const float4& self, float density, float vx,
                                                float vy, float vz, float pressure, float fx, float fy, float fz,
                                                uint32_t i, float4* __restrict__ pos_out,
                                                float4* __restrict__ vel_out, float4 learned) {
    // The force-field sum starts at vec3{0} and is added even when there are
    // no fields, which maps -0 to +0. A learned correction, when present, is
    // one more acceleration term; +0 leaves the plain step's bits unchanged.
    const float dt = __ldg(&t->dt);
    // Force fields (when the tank has any) were summed at the substep's start
    // positions by fields_kernel; otherwise the sum is the +0 of vec3{0}.
    float4 field = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (__ldg(&t->field_count) != 0) {
        field = __ldg(&t->field_accel[i]);
    }
    float ax = __fadd_rn(__fadd_rn(__fadd_rn(__fdiv_rn(fx, density), __ldg(&t->gravity[0])), field.x), learned.x);
    float ay = __fadd_rn(__fadd_rn(__fadd_rn(__fdiv_rn(fy, density), __ldg(&t->gravity[1])), field.y), learned.y);
    float az = __fadd_rn(__fadd_rn(__fadd_rn(__fdiv_rn(fz, density), __ldg(&t->gravity[2])), field.z), learned.z);
    vx = __fadd_rn(vx, __fmul_rn(ax, dt));
    vy = __fadd_rn(vy, __fmul_rn(ay, dt));
    vz = __fadd_rn(vz, __fmul_rn(az, dt));
    const float max_speed = __ldg(&t->max_speed);
    float speed = __fsqrt_rn(dot3(vx, vy, vz));
    if (speed > max_speed) {
        float s = __fdiv_rn(max_speed, speed);
        vx = __fmul_rn(vx, s);
        vy = __fmul_rn(vy, s);
        vz = __fmul_rn(vz, s);
    }
    float pp[3] = {__fadd_rn(self.x, __fmul_rn(vx, dt)), __fadd_rn(self.y, __fmul_rn(vy, dt)),
                   __fadd_rn(self.z, __fmul_rn(vz, dt))};
    float vv[3] = {vx, vy, vz};
    const float restitution = __ldg(&t->restitution);
#pragma unroll
    for (int axis = 0; axis < 3; ++axis) {
        float low = __ldg(&t->low[axis]);
        float high = __ldg(&t->high[axis]);
        if (pp[axis] < low) {
            pp[axis] = low;
            if (vv[axis] < 0.0f) {
                vv[axis] = __fmul_rn(-vv[axis], restitution);
            }
        } else if (pp[axis] > high) {
            pp[axis] = high;
            if (vv[axis] > 0.0f) {
                vv[axis] = __fmul_rn(-vv[axis], restitution);
            }
        }
    }
    pos_out[i] = make_float4(pp[0], pp[1], pp[2], density);
    vel_out[i] = make_float4(vv[0], vv[1], vv[2], pressure);
}

// Integrate in two phases per lane. The scan walks the candidate stream and
// keeps only in-range pairs, testing r^2 against the thresholds whose square
// roots round to h and 1e-6 (so `distance >= h || distance <= 1e-6` needs no
// square root per candidate); their sorted positions queue up in shared
// memory in stream order. When any lane's queue fills, the whole warp drains
// its queues, so the long per-pair force code runs with all lanes busy
// instead of once per candidate with most lanes masked off. Forces still add
// in the reference's order.
template <int kQueue>
__global__ void integrate_queued_kernel(const float4* __restrict__ spos2, const float4* __restrict__ svel,
                                        const uint32_t* __restrict__ sorted_ids, const uint2* __restrict__ bucket,
                                        const TankConst* __restrict__ tanks, const uint16_t* __restrict__ stank,
                                        uint32_t n, const uint32_t* __restrict__ order, float4* __restrict__ pos_out, float4* __restrict__ vel_out) {
    extern __shared__ uint32_t queue_smem[];
    uint32_t* queue = queue_smem + threadIdx.x;
    const uint32_t stride = blockDim.x;
    uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (order != nullptr && p < n) {
        p = order[p];
    }
    bool valid = p < n;
    const TankConst* t = tanks + (valid && stank != nullptr ? stank[p] : 0);
    valid = valid && __ldg(&t->active) != 0;
    PairConst k;
    k.h = __ldg(&t->h);
    k.c_spiky = __ldg(&t->c_spiky);
    k.c_visc = __ldg(&t->c_visc);
    k.neg_mass = __ldg(&t->neg_mass);
    k.visc_mass = __ldg(&t->visc_mass);
    const float r2_far = __ldg(&t->r2_far);
    const float r2_near = __ldg(&t->r2_near);
    const uint32_t mask = __ldg(&t->cell_mask);
    const uint32_t base = __ldg(&t->bucket_base);

    const float4 self = valid ? spos2[p] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    const float4 self_vel = valid ? svel[p] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    const uint32_t cx = static_cast<uint32_t>(cell_coord(self.x, k.h));
    const uint32_t cy = static_cast<uint32_t>(cell_coord(self.y, k.h));
    const uint32_t cz = static_cast<uint32_t>(cell_coord(self.z, k.h));
    float fx = 0.0f;
    float fy = 0.0f;
    float fz = 0.0f;
    uint32_t b = valid ? 0u : 27u;
    uint32_t cur = 0;
    uint32_t end = 0;
    uint32_t queued = 0;
    for (;;) {
        while (cur == end && b < 27u) {
            uint2 r = neighbour_range(bucket, cx, cy, cz, b, mask, base);
            cur = r.x;
            end = r.y;
            ++b;
        }
        bool has = cur < end;
        if (!__any_sync(0xFFFFFFFFu, has)) {
            break;
        }
        if (has) {
            float4 other = __ldg(&spos2[cur]);
            float ex = __fsub_rn(self.x, other.x);
            float ey = __fsub_rn(self.y, other.y);
            float ez = __fsub_rn(self.z, other.z);
            float r2 = dot3(ex, ey, ez);
            // Kept exactly when j != i and !(sqrt(r2) >= h || sqrt(r2) <= 1e-6).
            if (cur != p && !(r2 >= r2_far || r2 <= r2_near)) {
                queue[queued * stride] = cur;
                ++queued;
            }
            ++cur;
        }
        if (__any_sync(0xFFFFFFFFu, queued == static_cast<uint32_t>(kQueue))) {
            for (uint32_t e = 0; e < queued; ++e) {
                uint32_t q = queue[e * stride];
                add_pair_force(k, self, self_vel.x, self_vel.y, self_vel.z, self_vel.w, __ldg(&spos2[q]),
                               __ldg(&svel[q]), fx, fy, fz);
            }
            queued = 0;
        }
    }
    for (uint32_t e = 0; e < queued; ++e) {
        uint32_t q = queue[e * stride];
        add_pair_force(k, self, self_vel.x, self_vel.y, self_vel.z, self_vel.w, __ldg(&spos2[q]), __ldg(&svel[q]),
                       fx, fy, fz);
    }
    if (!valid) {
        return;
    }
    finish_particle(t, self, max_like_std(self.w, 1e-6f), self_vel.x, self_vel.y, self_vel.z, self_vel.w, fx, fy, fz,
                    sorted_ids[p], pos_out, vel_out);
}

// FluidSolver::emit (fluid_sph.cpp:138-154); glm's mat4 * vec4 adds the
// scaled columns as (c0 x + c1 y) + (c2 z + c3 w).
__global__ void emit_kernel(const TankConst* __restrict__ tank, uint32_t first, uint32_t count,
                            float4* __restrict__ pos, float4* __restrict__ vel, float4* __restrict__ prev) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) {
        return;
    }
    uint32_t cxn = max(tank->lattice[0], 1u);
    uint32_t cyn = max(tank->lattice[1], 1u);
    uint32_t czn = max(tank->lattice[2], 1u);
    float s = tank->spacing;
    uint32_t index[3] = {i % cxn, (i / cxn) % cyn, i / (cxn * cyn)};
    uint32_t counts[3] = {cxn, cyn, czn};
    float local[4];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        float extent = __fmul_rn(__fmul_rn(static_cast<float>(counts[a] - 1u), s), 0.5f);
        local[a] = __fsub_rn(__fmul_rn(static_cast<float>(index[a]), s), extent);
    }
    local[3] = 1.0f;
    const float* m = tank->emitter_world;
    float world[3];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        float add0 = __fadd_rn(__fmul_rn(m[0 * 4 + r], local[0]), __fmul_rn(m[1 * 4 + r], local[1]));
        float add1 = __fadd_rn(__fmul_rn(m[2 * 4 + r], local[2]), __fmul_rn(m[3 * 4 + r], local[3]));
        world[r] = __fadd_rn(add0, add1);
    }
    pos[first + i] = make_float4(world[0], world[1], world[2], tank->rest_w);
    vel[first + i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    prev[first + i] = make_float4(world[0], world[1], world[2], 0.0f);
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        v += __shfl_down_sync(0xFFFFFFFFu, v, o);
    }
    return v;
}

__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        v = fmax(v, __shfl_down_sync(0xFFFFFFFFu, v, o));
    }
    return v;
}

// Per-tank FP64 sums. Block b takes a contiguous range of particles (a
// multiple of 32), so a warp's consecutive 32-particle iterations mostly stay
// in one tank: each lane adds its particles into FP64 registers, and the warp
// reduces them with shuffles and adds them to the tank's accumulators only
// when its tank changes, and at the end. An iteration whose lanes straddle
// two tanks (or run past the range) is added on its own, per tank.
__device__ __forceinline__ void stats_terms(const float4* __restrict__ pos, const float4* __restrict__ vel,
                                            const TankConst* __restrict__ t, uint32_t i, double* v) {
    const float4 p = pos[i];
    const float4 u = vel[i];
    const double rho0 = t->rest_density;
    const double rho = p.w;
    const bool finite =
        isfinite(p.x) && isfinite(p.y) && isfinite(p.z) && isfinite(u.x) && isfinite(u.y) && isfinite(u.z);
    v[0] = rho;
    v[1] = fmax(0.0, rho - rho0) * (1.0 / rho0);
    v[2] = rho;
    v[3] = p.x;
    v[4] = p.y;
    v[5] = p.z;
    v[6] = 0.5 * static_cast<double>(t->mass) *
           (static_cast<double>(u.x) * u.x + static_cast<double>(u.y) * u.y + static_cast<double>(u.z) * u.z);
    v[7] = finite ? 0.0 : 1.0;
    v[8] = 1.0;
}

__device__ __forceinline__ void stats_add(double* dst, const double* s) {
#pragma unroll
    for (int k = 0; k < static_cast<int>(kStatsPerTank); ++k) {
        if (k == 2) {
            atomicMax(reinterpret_cast<unsigned long long*>(dst + 2),
                      static_cast<unsigned long long>(__double_as_longlong(fmax(s[2], 0.0))));
        } else if (k != 9) {
            atomicAdd(dst + k, s[k]);
        }
    }
}

__global__ void __launch_bounds__(256) stats_kernel(const float4* __restrict__ pos, const float4* __restrict__ vel,
                                                    const uint16_t* __restrict__ tank_of,
                                                    const TankConst* __restrict__ tanks, uint32_t n,
                                                    double* __restrict__ acc) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t warp = threadIdx.x >> 5;
    const size_t per_block = ((static_cast<size_t>(n) + gridDim.x - 1) / gridDim.x + 31) & ~static_cast<size_t>(31);
    const size_t begin = blockIdx.x * per_block;
    const size_t end = begin + per_block < n ? begin + per_block : n;
    double s[kStatsPerTank];
#pragma unroll
    for (int k = 0; k < static_cast<int>(kStatsPerTank); ++k) {
        s[k] = 0.0;
    }
    uint32_t current = 0xFFFFFFFFu;  // the tank the lanes' partial sums belong to (warp-uniform)
    auto flush = [&]() {
        if (current == 0xFFFFFFFFu) {
            return;
        }
        double r[kStatsPerTank];
#pragma unroll
        for (int k = 0; k < static_cast<int>(kStatsPerTank); ++k) {
            r[k] = k == 2 ? warp_max(s[k]) : warp_sum(s[k]);
            s[k] = 0.0;
        }
        if (lane == 0) {
            stats_add(acc + static_cast<size_t>(current) * kStatsPerTank, r);
        }
    };
    for (size_t first = begin + 32u * warp; first < end; first += blockDim.x) {
        const size_t idx = first + lane;
        const bool valid = idx < end;
        const uint32_t i = static_cast<uint32_t>(valid ? idx : 0);
        const uint32_t key = valid ? (tank_of != nullptr ? tank_of[i] : 0u) : 0xFFFFFFFFu;
        const uint32_t lead = __shfl_sync(0xFFFFFFFFu, key, 0);
        if (__all_sync(0xFFFFFFFFu, key == lead)) {
            // All 32 lanes hold particles of one tank: accumulate.
            if (lead != current) {
                flush();
                current = lead;
            }
            double v[kStatsPerTank];
            stats_terms(pos, vel, tanks + lead, i, v);
#pragma unroll
            for (int k = 0; k < static_cast<int>(kStatsPerTank); ++k) {
                s[k] = k == 2 ? fmax(s[k], v[k]) : s[k] + v[k];
            }
        } else {
            // Lanes of several tanks, or past the range: per tank, now.
            double v[kStatsPerTank];
#pragma unroll
            for (int k = 0; k < static_cast<int>(kStatsPerTank); ++k) {
                v[k] = 0.0;
            }
            if (valid) {
                stats_terms(pos, vel, tanks + key, i, v);
            }
            const uint32_t peers = __match_any_sync(0xFFFFFFFFu, key);
            if (valid) {
                // Reduce within the lanes of this tank, in lane order.
                double r[kStatsPerTank];
#pragma unroll
                for (int k = 0; k < static_cast<int>(kStatsPerTank); ++k) {
                    r[k] = 0.0;
                }
                uint32_t m = peers;
                while (m != 0) {
                    const int src = __ffs(m) - 1;
                    m &= m - 1;
#pragma unroll
                    for (int k = 0; k < static_cast<int>(kStatsPerTank); ++k) {
                        const double x = __shfl_sync(peers, v[k], src);
                        r[k] = k == 2 ? fmax(r[k], x) : r[k] + x;
                    }
                }
                if (lane == static_cast<uint32_t>(__ffs(peers) - 1)) {
                    stats_add(acc + static_cast<size_t>(key) * kStatsPerTank, r);
                }
            }
        }
    }
    flush();
}

__global__ void nonfinite_kernel(const float4* __restrict__ pos, const float4* __restrict__ vel, uint32_t n,
                                 uint32_t* __restrict__ out) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    bool bad = false;
    if (i < n) {
        float4 p = pos[i];
        float4 v = vel[i];
        bad = !(isfinite(p.x) && isfinite(p.y) && isfinite(p.z) && isfinite(v.x) && isfinite(v.y) && isfinite(v.z));
    }
    uint32_t votes = __ballot_sync(0xFFFFFFFFu, bad);
    if ((threadIdx.x & 31) == 0 && votes != 0) {
        atomicAdd(out, static_cast<uint32_t>(__popc(votes)));
    }
}

__global__ void bucket_stats_kernel(const uint2* __restrict__ bucket, uint32_t buckets, uint32_t* __restrict__ out) {
    uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t count = 0;
    if (b < buckets) {
        uint2 r = bucket[b];
        count = r.y - r.x;
    }
    uint32_t mx = count;
    uint32_t over = count > kCellCapacity ? 1u : 0u;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        mx = max(mx, __shfl_down_sync(0xFFFFFFFFu, mx, o));
        over += __shfl_down_sync(0xFFFFFFFFu, over, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMax(out, mx);
        atomicAdd(out + 1, over);
    }
}

// ---- list-driven variant ---------------------------------------------------
//
// Density walks the candidate stream two candidates at a time with packed
// f32x2 arithmetic (each lane of a packed add/sub/mul is rounded like the
// scalar operation) and adds the poly6 terms without branches: a candidate
// out of range adds +0, which leaves the non-negative running sum unchanged,
// so the sum is the reference's bit for bit. On the same pass it records, per
// particle, which candidates integrate will use (j != i and
// !(sqrt(r2) >= h || sqrt(r2) <= 1e-6), tested on r2 against exact square-root
// thresholds), as 16-bit codes (bucket index << 5 | slot) in stream order.
// Integrate then runs only the recorded pairs, so every lane of a warp spends
// its time in the force code instead of in a candidate scan where most lanes
// idle. A particle with more pairs than the list holds is flagged and
// integrate scans its candidates directly (same order, same bits).

__device__ __forceinline__ unsigned long long pack2(float a, float b) {
    unsigned long long r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}

__device__ __forceinline__ void unpack2(unsigned long long v, float& a, float& b) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v));
}

__device__ __forceinline__ unsigned long long sub2(unsigned long long a, unsigned long long b) {
    unsigned long long r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}

__device__ __forceinline__ unsigned long long add2(unsigned long long a, unsigned long long b) {
    unsigned long long r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}

__device__ __forceinline__ unsigned long long mul2(unsigned long long a, unsigned long long b) {
    unsigned long long r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}

template <bool kCount, bool kPacked>
__global__ void __launch_bounds__(128) density_list_kernel(const float4* __restrict__ spos, float4* __restrict__ svel,
                                                           float4* __restrict__ spos2, const uint2* __restrict__ bucket,
                                                           const TankConst* __restrict__ tanks,
                                                           const uint16_t* __restrict__ stank, uint32_t n, const uint32_t* __restrict__ order,
                                                           uint16_t* __restrict__ pair_list,
                                                           uint16_t* __restrict__ pair_count, uint32_t cap,
                                                           StepCounters* __restrict__ counters) {
    const uint32_t slot = blockIdx.x * blockDim.x + threadIdx.x;  // processing slot: indexes the masks
    uint32_t p = slot;
    if (order != nullptr && p < n) {
        p = order[p];
    }
    if (p >= n) {
        return;
    }
    const TankConst* t = tanks + (stank != nullptr ? stank[p] : 0);
    const float h = __ldg(&t->h);
    const float h2 = __ldg(&t->h2);
    const float r2_far = __ldg(&t->r2_far);
    const float r2_near = __ldg(&t->r2_near);
    const uint32_t mask = __ldg(&t->cell_mask);
    const uint32_t base = __ldg(&t->bucket_base);
    const float c6 = __ldg(&t->c_poly6);
    const float mass = __ldg(&t->mass);
    const unsigned long long h2x2 = pack2(h2, h2);
    const unsigned long long c6x2 = pack2(c6, c6);
    const unsigned long long massx2 = pack2(mass, mass);
    const float4 self = spos[p];
    const unsigned long long sx = pack2(self.x, self.x);
    const unsigned long long sy = pack2(self.y, self.y);
    const unsigned long long sz = pack2(self.z, self.z);
    const uint32_t cx = static_cast<uint32_t>(cell_coord(self.x, h));
    const uint32_t cy = static_cast<uint32_t>(cell_coord(self.y, h));
    const uint32_t cz = static_cast<uint32_t>(cell_coord(self.z, h));
    uint16_t* list = pair_list + static_cast<size_t>(p) * cap;
    float density = 0.0f;
    uint32_t listed = 0;
    uint32_t candidates = 0;
    uint32_t in_range = 0;
    for (uint32_t b = 0; b < 27u; ++b) {
        uint2 r = neighbour_range(bucket, cx, cy, cz, b, mask, base);
        uint32_t count = r.y - r.x;
        if (kCount) {
            candidates += count;
        }
        for (uint32_t k = 0; k < count; k += 2) {
            uint32_t qa = r.x + k;
            bool has_b = k + 1 < count;
            uint32_t qb = has_b ? qa + 1 : qa;
            float4 oa = __ldg(&spos[qa]);
            float4 ob = __ldg(&spos[qb]);
            float r2a, r2b, wa, wb;
            if constexpr (kPacked) {
                unsigned long long ex = sub2(sx, pack2(oa.x, ob.x));
                unsigned long long ey = sub2(sy, pack2(oa.y, ob.y));
                unsigned long long ez = sub2(sz, pack2(oa.z, ob.z));
                unsigned long long r2 = add2(add2(mul2(ex, ex), mul2(ey, ey)), mul2(ez, ez));
                unsigned long long d = sub2(h2x2, r2);
                unsigned long long w = mul2(massx2, mul2(mul2(mul2(c6x2, d), d), d));
                unpack2(r2, r2a, r2b);
                unpack2(w, wa, wb);
            } else {
                r2a = dot3(__fsub_rn(self.x, oa.x), __fsub_rn(self.y, oa.y), __fsub_rn(self.z, oa.z));
                r2b = dot3(__fsub_rn(self.x, ob.x), __fsub_rn(self.y, ob.y), __fsub_rn(self.z, ob.z));
                float da = __fsub_rn(h2, r2a);
                float db = __fsub_rn(h2, r2b);
                wa = __fmul_rn(mass, __fmul_rn(__fmul_rn(__fmul_rn(c6, da), da), da));
                wb = __fmul_rn(mass, __fmul_rn(__fmul_rn(__fmul_rn(c6, db), db), db));
            }
            bool in_a = r2a < h2;
            bool in_b = has_b && r2b < h2;
            density = __fadd_rn(density, in_a ? wa : 0.0f);
            density = __fadd_rn(density, in_b ? wb : 0.0f);
            if (kCount) {
                in_range += (in_a ? 1u : 0u) + (in_b ? 1u : 0u);
            }
            bool keep_a = qa != p && !(r2a >= r2_far || r2a <= r2_near);
            bool keep_b = has_b && qb != p && !(r2b >= r2_far || r2b <= r2_near);
            if (keep_a) {
                if (listed < cap) {
                    list[listed] = static_cast<uint16_t>((b << 5) | k);
                }
                ++listed;
            }
            if (keep_b) {
                if (listed < cap) {
                    list[listed] = static_cast<uint16_t>((b << 5) | (k + 1));
                }
                ++listed;
            }
        }
    }
    pair_count[p] = static_cast<uint16_t>(min(listed, 0xFFFFu));
    if (kCount) {
        unsigned long long c = candidates;
        unsigned long long rr = in_range;
        unsigned int active = __activemask();
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            c += __shfl_down_sync(active, c, o);
            rr += __shfl_down_sync(active, rr, o);
        }
        if ((threadIdx.x & 31) == static_cast<uint32_t>(__ffs(active) - 1)) {
            atomicAdd(&counters->candidates, c);
            atomicAdd(&counters->in_range, rr);
        }
    }
    density = max_like_std(density, 1e-6f);
    float pressure =
        max_like_std(__fmul_rn(__ldg(&t->stiffness), __fsub_rn(density, __ldg(&t->rest_density))), 0.0f);
    spos2[p] = make_float4(self.x, self.y, self.z, density);
    reinterpret_cast<float*>(svel)[4 * static_cast<size_t>(p) + 3] = pressure;
}


// Intermediates of one pair that the learned step's features reuse.
struct PairParts {
    float ex, ey, ez;  // x_i - x_j
    float distance;
    float dvx, dvy, dvz;  // v_j - v_i
};

// Pair force with the two shared reciprocals (1/distance, 1/rho_j); the same
// operations and order as add_pair_force. `parts` receives the offset,
// distance and velocity difference it computed on the way.
__device__ __forceinline__ void add_pair_force_rcp(const PairConst& k, const float4& self, float vx, float vy, float vz,
                                                   float pressure, const float4& other, const float4& ov, float& fx,
                                                   float& fy, float& fz, PairParts& parts) {
    float ex = __fsub_rn(self.x, other.x);
    float ey = __fsub_rn(self.y, other.y);
    float ez = __fsub_rn(self.z, other.z);
    float distance = __fsqrt_rn(dot3(ex, ey, ez));
    float inv_distance = __frcp_rn(distance);
    float other_density = max_like_std(other.w, 1e-6f);
    float inv_density = __frcp_rn(other_density);
    // 1 / (2 rho_j) is RN(1/rho_j) / 2 exactly (a power-of-two scaling).
    float ps = div_by(__fmul_rn(k.neg_mass, __fadd_rn(pressure, ov.w)), __fmul_rn(2.0f, other_density),
                      __fmul_rn(0.5f, inv_density));
    float d = __fsub_rn(k.h, distance);
    float gs = __fmul_rn(__fmul_rn(k.c_spiky, d), d);
    fx = __fadd_rn(fx, __fmul_rn(ps, __fmul_rn(gs, div_by(ex, distance, inv_distance))));
    fy = __fadd_rn(fy, __fmul_rn(ps, __fmul_rn(gs, div_by(ey, distance, inv_distance))));
    fz = __fadd_rn(fz, __fmul_rn(ps, __fmul_rn(gs, div_by(ez, distance, inv_distance))));
    float lap = __fmul_rn(k.c_visc, d);
    const float dvx = __fsub_rn(ov.x, vx);
    const float dvy = __fsub_rn(ov.y, vy);
    const float dvz = __fsub_rn(ov.z, vz);
    fx = __fadd_rn(fx, __fmul_rn(div_by(__fmul_rn(k.visc_mass, dvx), other_density, inv_density), lap));
    fy = __fadd_rn(fy, __fmul_rn(div_by(__fmul_rn(k.visc_mass, dvy), other_density, inv_density), lap));
    fz = __fadd_rn(fz, __fmul_rn(div_by(__fmul_rn(k.visc_mass, dvz), other_density, inv_density), lap));
    parts.ex = ex;
    parts.ey = ey;
    parts.ez = ez;
    parts.distance = distance;
    parts.dvx = dvx;
    parts.dvy = dvy;
    parts.dvz = dvz;
}

__device__ __forceinline__ void add_pair_force_rcp(const PairConst& k, const float4& self, float vx, float vy, float vz,
                                                   float pressure, const float4& other, const float4& ov, float& fx,
                                                   float& fy, float& fz) {
    PairParts unused;
    add_pair_force_rcp(k, self, vx, vy, vz, pressure, other, ov, fx, fy, fz, unused);
}

template <int kBlock, bool kRcp>
__global__ void __launch_bounds__(kBlock) integrate_list_kernel(const float4* __restrict__ spos2,
                                                                const float4* __restrict__ svel,
                                                                const uint32_t* __restrict__ sorted_ids,
                                                                const uint2* __restrict__ bucket,
                                                                const TankConst* __restrict__ tanks,
                                                                const uint16_t* __restrict__ stank, uint32_t n, const uint32_t* __restrict__ order,
                                                                const uint16_t* __restrict__ pair_list,
                                                                const uint16_t* __restrict__ pair_count, uint32_t cap,
                                                                float4* __restrict__ pos_out,
                                                                float4* __restrict__ vel_out) {
    __shared__ uint32_t starts[27][kBlock];
    uint32_t p = blockIdx.x * kBlock + threadIdx.x;
    if (order != nullptr && p < n) {
        p = order[p];
    }
    if (p >= n) {
        return;
    }
    const TankConst* t = tanks + (stank != nullptr ? stank[p] : 0);
    if (__ldg(&t->active) == 0) {
        return;
    }
    PairConst k;
    k.h = __ldg(&t->h);
    k.c_spiky = __ldg(&t->c_spiky);
    k.c_visc = __ldg(&t->c_visc);
    k.neg_mass = __ldg(&t->neg_mass);
    k.visc_mass = __ldg(&t->visc_mass);
    const uint32_t mask = __ldg(&t->cell_mask);
    const uint32_t base = __ldg(&t->bucket_base);
    const float4 self = spos2[p];
    const float4 self_vel = svel[p];
    const uint32_t cx = static_cast<uint32_t>(cell_coord(self.x, k.h));
    const uint32_t cy = static_cast<uint32_t>(cell_coord(self.y, k.h));
    const uint32_t cz = static_cast<uint32_t>(cell_coord(self.z, k.h));
    float fx = 0.0f;
    float fy = 0.0f;
    float fz = 0.0f;
    uint32_t pairs = pair_count[p];
    if (pairs <= cap) {
        for (uint32_t b = 0; b < 27u; ++b) {
            starts[b][threadIdx.x] = neighbour_range(bucket, cx, cy, cz, b, mask, base).x;
        }
        const uint16_t* list = pair_list + static_cast<size_t>(p) * cap;
        for (uint32_t e = 0; e < pairs; ++e) {
            uint32_t code = list[e];
            uint32_t q = starts[code >> 5][threadIdx.x] + (code & 31u);
            if (kRcp) {
                add_pair_force_rcp(k, self, self_vel.x, self_vel.y, self_vel.z, self_vel.w, __ldg(&spos2[q]),
                                   __ldg(&svel[q]), fx, fy, fz);
            } else {
                add_pair_force(k, self, self_vel.x, self_vel.y, self_vel.z, self_vel.w, __ldg(&spos2[q]),
                               __ldg(&svel[q]), fx, fy, fz);
            }
        }
    } else {
        // More pairs than the list holds: scan the candidates (rare).
        const float r2_far = __ldg(&t->r2_far);
        const float r2_near = __ldg(&t->r2_near);
        for (uint32_t b = 0; b < 27u; ++b) {
            uint2 r = neighbour_range(bucket, cx, cy, cz, b, mask, base);
            for (uint32_t q = r.x; q < r.y; ++q) {
                float4 other = __ldg(&spos2[q]);
                float r2 = dot3(__fsub_rn(self.x, other.x), __fsub_rn(self.y, other.y), __fsub_rn(self.z, other.z));
                if (q != p && !(r2 >= r2_far || r2 <= r2_near)) {
                    if (kRcp) {
                        add_pair_force_rcp(k, self, self_vel.x, self_vel.y, self_vel.z, self_vel.w, other,
                                           __ldg(&svel[q]), fx, fy, fz);
                    } else {
                        add_pair_force(k, self, self_vel.x, self_vel.y, self_vel.z, self_vel.w, other,
                                       __ldg(&svel[q]), fx, fy, fz);
                    }
                }
            }
        }
    }
    finish_particle(t, self, max_like_std(self.w, 1e-6f), self_vel.x, self_vel.y, self_vel.z, self_vel.w, fx, fy, fz,
                    sorted_ids[p], pos_out, vel_out);
}

// ---- mask-driven variant ---------------------------------------------------
//
// Density keeps the nested bucket loops (all lanes of a warp step through the
// 27 buckets together) and, per bucket, ORs into one 32-bit word the slots
// integrate will use (j != i and !(sqrt(r2) >= h || sqrt(r2) <= 1e-6), via the
// exact r2 thresholds). The word is stored bucket-major by processing slot,
// masks[b * n + slot], so each store of a warp is one contiguous 128-byte line
// whatever the processing order. Integrate reads its 27
// words (again one line per warp and bucket), expands the set bits into a
// list of sorted positions in shared memory in stream order, and runs the
// pair forces over that list with all lanes busy.
template <bool kCount>
__global__ void __launch_bounds__(128) density_mask_kernel(const float4* __restrict__ spos, float4* __restrict__ svel,
                                                           float4* __restrict__ spos2, const uint2* __restrict__ bucket,
                                                           const TankConst* __restrict__ tanks,
                                                           const uint16_t* __restrict__ stank, uint32_t n, const uint32_t* __restrict__ order,
                                                           uint32_t* __restrict__ masks,
                                                           StepCounters* __restrict__ counters, int all_tanks) {
    const uint32_t slot = blockIdx.x * blockDim.x + threadIdx.x;  // processing slot: indexes the masks
    uint32_t p = slot;
    if (order != nullptr && p < n) {
        p = order[p];
    }
    if (p >= n) {
        return;
    }
    const TankConst* t = tanks + (stank != nullptr ? stank[p] : 0);
    // A tank that sits this substep out is not integrated, and tanks never
    // share pairs, so its densities are not needed (pair counting visits all).
    if (!kCount && all_tanks == 0 && __ldg(&t->active) == 0) {
        return;
    }
    const float h = __ldg(&t->h);
    const float h2 = __ldg(&t->h2);
    const float c6 = __ldg(&t->c_poly6);
    const float mass = __ldg(&t->mass);
    const float r2_far = __ldg(&t->r2_far);
    const float r2_near = __ldg(&t->r2_near);
    const uint32_t cell_mask = __ldg(&t->cell_mask);
    const uint32_t base = __ldg(&t->bucket_base);
    const float4 self = spos[p];
    const uint32_t cx = static_cast<uint32_t>(cell_coord(self.x, h));
    const uint32_t cy = static_cast<uint32_t>(cell_coord(self.y, h));
    const uint32_t cz = static_cast<uint32_t>(cell_coord(self.z, h));
    float density = 0.0f;
    uint32_t candidates = 0;
    uint32_t in_range = 0;
    // kMax: out-of-range terms are dropped by max.NaN(term, +0), valid while
    // mass * c_poly6 > 0 (then out of range, where d <= 0, the term is negative
    // or +0); otherwise by the reference's compare and select.
    auto walk = [&](auto max_form) {
        constexpr bool kMax = decltype(max_form)::value;
        for (uint32_t b = 0; b < 27u; ++b) {
            uint2 r = neighbour_range(bucket, cx, cy, cz, b, cell_mask, base);
            uint32_t word = 0;
            if (kCount) {
                candidates += r.y - r.x;
            }
            const float4* cand = spos + r.x;
            const uint32_t count = r.y - r.x;
            // Branch-free candidate loop: every lane runs the same instructions
            // for every candidate, so a warp issues each of them once.
#pragma unroll 2
            for (uint32_t s = 0; s < count; ++s) {
                float4 other = __ldg(&cand[s]);
                float r2 = dot3(__fsub_rn(self.x, other.x), __fsub_rn(self.y, other.y), __fsub_rn(self.z, other.z));
                // mass * poly6 (fluid_sph.cpp:24-31, :214) in candidate order;
                // out of range the reference adds mass * 0 = +0, which leaves
                // the (non-negative) sum's bits as they are, and a NaN distance
                // makes the sum NaN (max.NaN keeps it).
                float d = __fsub_rn(h2, r2);
                float term = __fmul_rn(mass, __fmul_rn(__fmul_rn(__fmul_rn(c6, d), d), d));
                float kept;
                if (kMax) {
                    asm("max.NaN.f32 %0, %1, %2;" : "=f"(kept) : "f"(term), "f"(0.0f));
                } else {
                    kept = r2 >= h2 ? 0.0f : term;
                }
                density = __fadd_rn(density, kept);
                if (kCount) {
                    in_range += r2 < h2 ? 1u : 0u;
                }
                // Integrate skips distance >= h or <= 1e-6 (fluid_sph.cpp:245-248);
                // the particle itself (r2 = 0) fails the second test. Slot s's
                // bit is shifted in s-th (no per-candidate shift count).
                word = (word << 1) | static_cast<uint32_t>(!(r2 >= r2_far || r2 <= r2_near));
            }
            // Reverse into place: bit s for slot s (count <= 32 slots).
            word = count == 0 ? 0u : (__brev(word) >> (32u - count));
            masks[static_cast<size_t>(b) * n + slot] = word;
        }
    };
    if (mass > 0.0f && c6 > 0.0f) {
        walk(std::true_type{});
    } else {
        walk(std::false_type{});
    }
    if (kCount) {
        unsigned long long c = candidates;
        unsigned long long rr = in_range;
        unsigned int active = __activemask();
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            c += __shfl_down_sync(active, c, o);
            rr += __shfl_down_sync(active, rr, o);
        }
        if ((threadIdx.x & 31) == static_cast<uint32_t>(__ffs(active) - 1)) {
            atomicAdd(&counters->candidates, c);
            atomicAdd(&counters->in_range, rr);
        }
    }
    density = max_like_std(density, 1e-6f);
    float pressure =
        max_like_std(__fmul_rn(__ldg(&t->stiffness), __fsub_rn(density, __ldg(&t->rest_density))), 0.0f);
    spos2[p] = make_float4(self.x, self.y, self.z, density);
    reinterpret_cast<float*>(svel)[4 * static_cast<size_t>(p) + 3] = pressure;
}

// kMinBlocks: resident blocks per SM the register budget must allow (128
// threads x 9 blocks = 36 warps at 56 registers, against 32 warps at the
// 57 registers the kernel takes unbounded, whose allocation rounds to 64).
// The default <128, 40, 9> lists 40 pairs per thread (20 KB of shared memory
// a block, 180 KB an SM): a compressed tank (about 40 pairs a particle) then
// rarely drains mid-walk, and L1 keeps 76 KB; 44 or 48 entries leave too
// little L1 and ran 8-20 % slower.
// kGroup: mask words and bucket starts loaded kGroup buckets at a time (27 % kGroup == 0).
template <int kBlock, int kList, int kMinBlocks = 1, uint32_t kGroup = 3>
__global__ void __launch_bounds__(kBlock, kMinBlocks) integrate_mask_kernel(const float4* __restrict__ spos2,
                                                                const float4* __restrict__ svel,
                                                                const uint32_t* __restrict__ sorted_ids,
                                                                const uint2* __restrict__ bucket,
                                                                const TankConst* __restrict__ tanks,
                                                                const uint16_t* __restrict__ stank, uint32_t n, const uint32_t* __restrict__ order,
                                                                const uint32_t* __restrict__ masks,
                                                                float4* __restrict__ pos_out,
                                                                float4* __restrict__ vel_out, uint32_t slots) {
    // One bucket may hand over 32 pairs at once, after the warp has drained.
    static_assert(kList >= 32, "a pair list must hold a whole bucket");
    static_assert(27u % kGroup == 0, "groups of buckets tile the 27");
    // A launch that follows this one programmatically (the next slot range,
    // which reads nothing this one writes) may start once every block of
    // this one has started: its blocks then fill this launch's tail.
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    __shared__ uint32_t list[kList][kBlock];
    // The launch's first `slots` processing slots (order and masks start at
    // the range's first slot; n stays the masks' row stride).
    const uint32_t slot = blockIdx.x * kBlock + threadIdx.x;
    bool valid = slot < slots;
    const uint32_t p = valid && order != nullptr ? order[slot] : slot;
    const TankConst* t = tanks + (valid && stank != nullptr ? stank[p] : 0);
    valid = valid && __ldg(&t->active) != 0;
    // The lanes with a particle; they walk the 27 buckets in step.
    const uint32_t live = __ballot_sync(0xFFFFFFFFu, valid);
    if (!valid) {
        return;
    }
    PairConst k;
    k.h = __ldg(&t->h);
    k.c_spiky = __ldg(&t->c_spiky);
    k.c_visc = __ldg(&t->c_visc);
    k.neg_mass = __ldg(&t->neg_mass);
    k.visc_mass = __ldg(&t->visc_mass);
    const uint32_t cell_mask = __ldg(&t->cell_mask);
    const uint32_t base = __ldg(&t->bucket_base);
    const float4 self = spos2[p];
    const float4 self_vel = svel[p];
    const uint32_t cx = static_cast<uint32_t>(cell_coord(self.x, k.h));
    const uint32_t cy = static_cast<uint32_t>(cell_coord(self.y, k.h));
    const uint32_t cz = static_cast<uint32_t>(cell_coord(self.z, k.h));
    float fx = 0.0f;
    float fy = 0.0f;
    float fz = 0.0f;
    uint32_t listed = 0;
    // kGroup buckets at a time: their mask words, then the first slots of the
    // buckets with pairs, are loaded back to back, so a particle waits for
    // two loads per group instead of two per bucket.
    for (uint32_t b0 = 0; b0 < 27u; b0 += kGroup) {
        uint32_t words[kGroup];
        uint32_t firsts[kGroup];
#pragma unroll
        for (uint32_t j = 0; j < kGroup; ++j) {
            words[j] = __ldg(&masks[static_cast<size_t>(b0 + j) * n + slot]);
        }
#pragma unroll
        for (uint32_t j = 0; j < kGroup; ++j) {
            firsts[j] = words[j] != 0 ? neighbour_range(bucket, cx, cy, cz, b0 + j, cell_mask, base).x : 0u;
        }
#pragma unroll
        for (uint32_t j = 0; j < kGroup; ++j) {
            uint32_t word = words[j];
            // When any lane's list cannot take this bucket's pairs, every lane
            // drains its list (in order) at once, so the force code runs with
            // all lanes busy rather than once per lane that filled up.
            if (__any_sync(live, listed + static_cast<uint32_t>(__popc(word)) > static_cast<uint32_t>(kList))) {
                for (uint32_t e = 0; e < listed; ++e) {
                    uint32_t q = list[e][threadIdx.x];
                    add_pair_force_rcp(k, self, self_vel.x, self_vel.y, self_vel.z, self_vel.w, __ldg(&spos2[q]),
                                       __ldg(&svel[q]), fx, fy, fz);
                }
                listed = 0;
            }
            while (word != 0) {
                uint32_t s = static_cast<uint32_t>(__ffs(word) - 1);
                word &= word - 1;
                list[listed][threadIdx.x] = firsts[j] + s;
                ++listed;
            }
        }
    }
    for (uint32_t e = 0; e < listed; ++e) {
        uint32_t q = list[e][threadIdx.x];
        add_pair_force_rcp(k, self, self_vel.x, self_vel.y, self_vel.z, self_vel.w, __ldg(&spos2[q]), __ldg(&svel[q]),
                           fx, fy, fz);
    }
    finish_particle(t, self, max_like_std(self.w, 1e-6f), self_vel.x, self_vel.y, self_vel.z, self_vel.w, fx, fy, fz,
                    sorted_ids[p], pos_out, vel_out);
}

// ---- shared-memory-staged integrate ----------------------------------------
//
// A block owns kThreads consecutive processing slots; in the Morton or
// Hilbert order they fill a compact run of cells, whose 27-bucket
// neighbourhoods overlap. Before any pair force the block copies the sorted
// position/density and velocity/pressure of every non-empty bucket its
// particles visit, each bucket once, into shared memory (cp.async, 16 bytes
// a lane, L1 bypassed), so the pairs read shared memory instead of gathering
// each neighbour through L1 and L2. Buckets are deduplicated by a shared
// hash table that one lane per run of same-cell lanes fills. A block whose
// buckets overflow the table or the data area reads global memory instead,
// with the same lists.
//
// Each lane lists its pairs from density's masks in (bucket, slot) order
// while the copies are in flight, up to kList of them; after the copies land
// it runs the list, then lists and runs the rest of its walk in list-sized
// rounds. The pairs go through add_pair_force_rcp in the reference's order,
// so every bit equals integrate_mask_kernel's (fluid_sph.cpp:234-258).

namespace staged {

constexpr uint32_t kEmptyKey = 0xFFFFFFFFu;  // bucket keys are below the bucket total (< 2^32 - 1)
constexpr uint32_t kSlack = 32;              // data entries past kCap: a bad list entry stays in bounds

__device__ __forceinline__ uint32_t table_slot(uint32_t key, uint32_t bits) {
    return (key * 0x9E3779B1u) >> (32u - bits);
}

__device__ __forceinline__ void copy16_async(void* dst_shared, const void* src_global) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(
                     static_cast<uint32_t>(__cvta_generic_to_shared(dst_shared))),
                 "l"(src_global)
                 : "memory");
}

__device__ __forceinline__ void copies_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// Global bucket index of neighbour b (the walk order of neighbour_range).
__device__ __forceinline__ uint32_t neighbour_key(uint32_t cx, uint32_t cy, uint32_t cz, uint32_t b, uint32_t mask,
                                                  uint32_t base) {
    const uint32_t dz = b / 9u;
    const uint32_t dy = (b / 3u) % 3u;
    const uint32_t dx = b % 3u;
    return base + spatial_hash(cx + dx - 1u, cy + dy - 1u, cz + dz - 1u, mask);
}

// Shared-memory layout (bytes). The region after the table holds the pair
// lists (u16 data indices, [kList][kThreads]); before them, while the table
// is built, it holds each slot's bucket start, count, the occupied slots in
// order and the scan's warp totals. The global-memory path keeps u32 lists
// in the (then unused) data area.
template <uint32_t kThreads, uint32_t kList, uint32_t kCap, uint32_t kTable>
struct Layout {
    static constexpr uint32_t kWarps = kThreads / 32u;
    static constexpr size_t kEntries = static_cast<size_t>(kCap) + kSlack;
    static constexpr size_t kPos = 0;
    static constexpr size_t kVel = kPos + kEntries * 16u;
    static constexpr size_t kKey = kVel + kEntries * 16u;
    static constexpr size_t kOff = kKey + static_cast<size_t>(kTable) * 4u;
    static constexpr size_t kRegion = kOff + static_cast<size_t>(kTable) * 2u;
    static constexpr size_t kStart = kRegion;
    static constexpr size_t kCnt = kStart + static_cast<size_t>(kTable) * 4u;
    static constexpr size_t kOcc = kCnt + static_cast<size_t>(kTable);
    static constexpr size_t kMisc = kOcc + static_cast<size_t>(kTable) * 2u;
    static constexpr size_t kBuildEnd = kMisc + (2u + kWarps) * 4u;
    static constexpr size_t kListEnd = kRegion + static_cast<size_t>(kList) * kThreads * 2u;
    static constexpr size_t kBytes = kBuildEnd > kListEnd ? kBuildEnd : kListEnd;
    static_assert(kThreads % 32u == 0 && kTable % kThreads == 0 && kTable % 4u == 0, "table split by thread");
    static_assert(kTable * kCellCapacity < 65536u, "scan packs entries and slots in one word");
    static_assert(kCap + kSlack <= 65536u, "data indices are 16-bit");
    static_assert(static_cast<size_t>(kList) * kThreads * 4u <= kEntries * 32u, "global lists fit the data area");
    static_assert(kList >= kCellCapacity, "a list takes a whole bucket");
};

}  // namespace staged

template <uint32_t kThreads, uint32_t kList, uint32_t kCap, uint32_t kTableBits, int kMinBlocks>
__global__ void __launch_bounds__(kThreads, kMinBlocks) integrate_staged_kernel(
    const float4* __restrict__ spos2, const float4* __restrict__ svel, const uint32_t* __restrict__ sorted_ids,
    const uint2* __restrict__ bucket, const TankConst* __restrict__ tanks, const uint16_t* __restrict__ stank,
    uint32_t n, const uint32_t* __restrict__ order, const uint32_t* __restrict__ masks, float4* __restrict__ pos_out,
    float4* __restrict__ vel_out) {
    constexpr uint32_t kTable = 1u << kTableBits;
    using L = staged::Layout<kThreads, kList, kCap, kTable>;
    constexpr uint32_t kPer = kTable / kThreads;
    extern __shared__ __align__(16) unsigned char smem[];
    float4* s_pos = reinterpret_cast<float4*>(smem + L::kPos);
    float4* s_vel = reinterpret_cast<float4*>(smem + L::kVel);
    uint32_t* s_key = reinterpret_cast<uint32_t*>(smem + L::kKey);
    uint16_t* s_off = reinterpret_cast<uint16_t*>(smem + L::kOff);
    uint16_t* s_list = reinterpret_cast<uint16_t*>(smem + L::kRegion);
    uint32_t* g_list = reinterpret_cast<uint32_t*>(smem + L::kPos);
    uint32_t* s_start = reinterpret_cast<uint32_t*>(smem + L::kStart);
    uint8_t* s_cnt = smem + L::kCnt;
    uint16_t* s_occ = reinterpret_cast<uint16_t*>(smem + L::kOcc);
    uint32_t* s_misc = reinterpret_cast<uint32_t*>(smem + L::kMisc);  // [0] table full, [2 + w] warp totals

    const uint32_t tid = threadIdx.x;
    const uint32_t lane = tid & 31u;
    const uint32_t warp = tid >> 5;
    const uint32_t slot = blockIdx.x * kThreads + tid;
    uint32_t p = slot;
    if (order != nullptr && p < n) {
        p = order[p];
    }
    bool valid = p < n;
    const uint32_t tank = valid && stank != nullptr ? stank[p] : 0u;
    const TankConst* t = tanks + tank;
    valid = valid && __ldg(&t->active) != 0;
    for (uint32_t i = tid; i < kTable; i += kThreads) {
        s_key[i] = staged::kEmptyKey;
        s_off[i] = 0;
    }
    if (tid == 0) {
        s_misc[0] = 0;
    }
    PairConst k{};
    uint32_t cell_mask = 0;
    uint32_t base = 0;
    uint32_t cx = 0;
    uint32_t cy = 0;
    uint32_t cz = 0;
    float4 self = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    float4 self_vel = self;
    if (valid) {
        k.h = __ldg(&t->h);
        k.c_spiky = __ldg(&t->c_spiky);
        k.c_visc = __ldg(&t->c_visc);
        k.neg_mass = __ldg(&t->neg_mass);
        k.visc_mass = __ldg(&t->visc_mass);
        cell_mask = __ldg(&t->cell_mask);
        base = __ldg(&t->bucket_base);
        self = spos2[p];
        self_vel = svel[p];
        cx = static_cast<uint32_t>(cell_coord(self.x, k.h));
        cy = static_cast<uint32_t>(cell_coord(self.y, k.h));
        cz = static_cast<uint32_t>(cell_coord(self.z, k.h));
    }
    __syncthreads();

    // 1. The first lane of each run of lanes in one cell (of one tank) enters
    //    the cell's non-empty buckets into the table.
    {
        const uint32_t pcx = __shfl_up_sync(0xFFFFFFFFu, cx, 1);
        const uint32_t pcy = __shfl_up_sync(0xFFFFFFFFu, cy, 1);
        const uint32_t pcz = __shfl_up_sync(0xFFFFFFFFu, cz, 1);
        const uint32_t ptank = __shfl_up_sync(0xFFFFFFFFu, tank, 1);
        const uint32_t vmask = __ballot_sync(0xFFFFFFFFu, valid);
        const bool prev_valid = lane > 0 && ((vmask >> (lane - 1u)) & 1u) != 0;
        const bool leader = valid && (!prev_valid || pcx != cx || pcy != cy || pcz != cz || ptank != tank);
        if (leader) {
            // Nine bucket ranges at a time, loaded back to back.
#pragma unroll
            for (uint32_t dz = 0; dz < 3u; ++dz) {
                uint32_t keys[9];
                uint2 ranges[9];
#pragma unroll
                for (uint32_t j = 0; j < 9u; ++j) {
                    keys[j] = staged::neighbour_key(cx, cy, cz, 9u * dz + j, cell_mask, base);
                    ranges[j] = __ldg(&bucket[keys[j]]);
                }
#pragma unroll
                for (uint32_t j = 0; j < 9u; ++j) {
                    const uint32_t key = keys[j];
                    const uint32_t cnt = min(ranges[j].y - ranges[j].x, kCellCapacity);
                    if (cnt == 0) {
                        continue;
                    }
                    uint32_t h = staged::table_slot(key, kTableBits);
                    uint32_t probe = 0;
                    for (; probe < kTable; ++probe) {
                        const uint32_t old = atomicCAS(&s_key[h], staged::kEmptyKey, key);
                        if (old == staged::kEmptyKey) {
                            s_start[h] = ranges[j].x;
                            s_cnt[h] = static_cast<uint8_t>(cnt);
                            break;
                        }
                        if (old == key) {
                            break;
                        }
                        h = (h + 1u) & (kTable - 1u);
                    }
                    if (probe == kTable) {
                        atomicOr(&s_misc[0], 1u);
                    }
                }
            }
        }
    }
    __syncthreads();

    // 2. Data offsets: a block-wide scan of (entries << 16 | slots) over the
    //    table, kPer consecutive slots a thread.
    uint32_t mine = 0;
#pragma unroll
    for (uint32_t j = 0; j < kPer; ++j) {
        const uint32_t s = tid * kPer + j;
        if (s_key[s] != staged::kEmptyKey) {
            mine += (static_cast<uint32_t>(s_cnt[s]) << 16) | 1u;
        }
    }
    uint32_t inclusive = mine;
#pragma unroll
    for (uint32_t o = 1; o < 32u; o <<= 1) {
        const uint32_t v = __shfl_up_sync(0xFFFFFFFFu, inclusive, o);
        if (lane >= o) {
            inclusive += v;
        }
    }
    if (lane == 31u) {
        s_misc[2u + warp] = inclusive;
    }
    __syncthreads();
    uint32_t before = inclusive - mine;
    uint32_t total = 0;
    for (uint32_t w = 0; w < L::kWarps; ++w) {
        const uint32_t v = s_misc[2u + w];
        before += w < warp ? v : 0u;
        total += v;
    }
    const uint32_t occupied = total & 0xFFFFu;
    // Block-uniform: every thread read the same words after the barrier.
    const bool staged_data = s_misc[0] == 0 && (total >> 16) <= kCap;
    if (staged_data) {
        uint32_t e = before >> 16;
        uint32_t o = before & 0xFFFFu;
#pragma unroll
        for (uint32_t j = 0; j < kPer; ++j) {
            const uint32_t s = tid * kPer + j;
            if (s_key[s] != staged::kEmptyKey) {
                s_off[s] = static_cast<uint16_t>(e);
                s_occ[o] = static_cast<uint16_t>(s);
                e += s_cnt[s];
                ++o;
            }
        }
    }
    __syncthreads();

    // 3. Copies: a warp per bucket, a lane per entry.
    if (staged_data) {
        for (uint32_t q = warp; q < occupied; q += L::kWarps) {
            const uint32_t s = s_occ[q];
            if (lane < s_cnt[s]) {
                const uint32_t src = s_start[s] + lane;
                const uint32_t dst = static_cast<uint32_t>(s_off[s]) + lane;
                staged::copy16_async(s_pos + dst, spos2 + src);
                staged::copy16_async(s_vel + dst, svel + src);
            }
        }
    }
    __syncthreads();  // the build arrays are dead: the region holds the lists now

    // 4. Lists and pairs. The first list comes from the 27 mask words loaded
    //    back to back; a walk longer than one list reloads the rest.
    uint32_t words[27];
#pragma unroll
    for (uint32_t b = 0; b < 27u; ++b) {
        words[b] = valid ? __ldg(&masks[static_cast<size_t>(b) * n + slot]) : 0u;
    }
    auto walk = [&](auto data_form) {
        constexpr bool kShared = decltype(data_form)::value;
        auto append = [&](uint32_t b, uint32_t word, uint32_t& listed) {
            const uint32_t key = staged::neighbour_key(cx, cy, cz, b, cell_mask, base);
            uint32_t first;
            if constexpr (kShared) {
                uint32_t h = staged::table_slot(key, kTableBits);
                for (uint32_t probe = 0; probe < kTable && s_key[h] != key; ++probe) {
                    h = (h + 1u) & (kTable - 1u);
                }
                first = s_off[h];
            } else {
                first = __ldg(&bucket[key]).x;
            }
            while (word != 0) {
                const uint32_t s = static_cast<uint32_t>(__ffs(word) - 1);
                word &= word - 1u;
                if constexpr (kShared) {
                    s_list[listed * kThreads + tid] = static_cast<uint16_t>(first + s);
                } else {
                    g_list[listed * kThreads + tid] = first + s;
                }
                ++listed;
            }
        };
        // The first list: buckets 0.. until one would not fit (b_next).
        auto fill_first = [&](uint32_t& b_next) -> uint32_t {
            uint32_t listed = 0;
            uint32_t stop = 27u;
#pragma unroll
            for (uint32_t b = 0; b < 27u; ++b) {
                const uint32_t word = words[b];
                if (stop != 27u || word == 0) {
                    continue;
                }
                if (listed + static_cast<uint32_t>(__popc(word)) > kList) {
                    stop = b;
                    continue;
                }
                append(b, word, listed);
            }
            b_next = stop;
            return listed;
        };
        // A later list: buckets b_next.. (masks reloaded).
        auto fill_rest = [&](uint32_t& b_next) -> uint32_t {
            uint32_t listed = 0;
            for (; b_next < 27u; ++b_next) {
                const uint32_t word = __ldg(&masks[static_cast<size_t>(b_next) * n + slot]);
                if (word == 0) {
                    continue;
                }
                if (listed + static_cast<uint32_t>(__popc(word)) > kList) {
                    break;
                }
                append(b_next, word, listed);
            }
            return listed;
        };
        float fx = 0.0f;
        float fy = 0.0f;
        float fz = 0.0f;
        auto run = [&](uint32_t listed) {
            for (uint32_t e = 0; e < listed; ++e) {
                if constexpr (kShared) {
                    const uint32_t q = s_list[e * kThreads + tid];
                    add_pair_force_rcp(k, self, self_vel.x, self_vel.y, self_vel.z, self_vel.w, s_pos[q], s_vel[q],
                                       fx, fy, fz);
                } else {
                    const uint32_t q = g_list[e * kThreads + tid];
                    add_pair_force_rcp(k, self, self_vel.x, self_vel.y, self_vel.z, self_vel.w, __ldg(&spos2[q]),
                                       __ldg(&svel[q]), fx, fy, fz);
                }
            }
        };
        uint32_t b = 27u;
        const uint32_t listed = valid ? fill_first(b) : 0u;
        if constexpr (kShared) {
            staged::copies_wait_all();
        }
        __syncthreads();  // every lane's copies have landed
        if (!valid) {
            return;
        }
        run(listed);
        while (b < 27u) {
            run(fill_rest(b));
        }
        finish_particle(t, self, max_like_std(self.w, 1e-6f), self_vel.x, self_vel.y, self_vel.z, self_vel.w, fx, fy,
                        fz, sorted_ids[p], pos_out, vel_out);
    };
    if (staged_data) {
        walk(std::true_type{});
    } else {
        walk(std::false_type{});
    }
}

// ---- cell-cooperative variant ------------------------------------------------
//
// A warp owns 32 consecutive processing slots. Consecutive slots whose
// particles lie in the same cell of the same tank form a group: a cell's
// particles are consecutive in the Morton processing order (in sorted order
// a bucket shared by two cells can split a cell into several groups, which
// costs time only). Every particle of a group has the same 27 neighbour
// buckets, so the group's candidates, the first min(count, 32) entries of
// each bucket concatenated in the reference's (dz, dy, dx) order
// (fluid_sph.cpp:205-216, :234-258), are listed once in shared memory and
// visited by all 32 lanes at once instead of once per particle.
//
// Density: lanes take 32 candidates at a time and loop over the group's
// particles. Each (particle, candidate) poly6 term goes to shared memory and
// the particle's own lane adds its row in candidate order; an out-of-range
// term is +0, which leaves the non-negative sum's bits as they are, so the
// sum is the reference's bit for bit. The same pass records which pairs
// integrate uses, one 32-bit word per particle and 32 candidates, stored
// chunk-major by processing slot (masks[c * n + slot]).
//
// Integrate: the group's pairs are computed in rounds. Each particle's lane
// lists its next pairs (in candidate order); all 32 lanes compute the
// pressure and viscosity terms of the listed pairs into shared memory, one
// pair per lane; then lanes that own one (particle, axis) add the terms in
// the reference's order. The forces, and so every result bit, are those of
// the per-particle kernels.

constexpr uint32_t kCoopWarps = 4;                             // warps per block
constexpr uint32_t kCoopMaxCandidates = 27u * kCellCapacity;  // 864
constexpr uint32_t kCoopMaxChunks = kCoopMaxCandidates / 32u;  // 27 mask words per particle at most
constexpr uint32_t kCoopPairs = 256;                           // pairs listed per integrate round
constexpr uint32_t kFullMask = 0xFFFFFFFFu;
static_assert(kCoopMaxChunks <= 27u, "the mask buffer holds 27 words per particle");

// Group starts of a window: lane l starts a group when it holds a particle
// and lane l - 1 holds none, or one of another cell or tank.
__device__ __forceinline__ uint32_t coop_group_starts(bool valid, uint32_t tank, uint32_t cx, uint32_t cy,
                                                      uint32_t cz, uint32_t lane, uint32_t& valid_mask) {
    const uint32_t pcx = __shfl_up_sync(kFullMask, cx, 1);
    const uint32_t pcy = __shfl_up_sync(kFullMask, cy, 1);
    const uint32_t pcz = __shfl_up_sync(kFullMask, cz, 1);
    const uint32_t ptank = __shfl_up_sync(kFullMask, tank, 1);
    valid_mask = __ballot_sync(kFullMask, valid);
    const bool prev_valid = lane > 0 && ((valid_mask >> (lane - 1u)) & 1u) != 0;
    const bool start = valid && (!prev_valid || pcx != cx || pcy != cy || pcz != cz || ptank != tank);
    return __ballot_sync(kFullMask, start);
}

// One past the last lane of the group that starts at lane s: the next group
// start or the first lane without a particle after s.
__device__ __forceinline__ uint32_t coop_group_end(uint32_t s, uint32_t later_starts, uint32_t valid_mask) {
    const uint32_t above = s >= 31u ? 0u : (kFullMask << (s + 1u));
    const uint32_t stop = (later_starts | ~valid_mask) & above;
    return stop == 0 ? 32u : static_cast<uint32_t>(__ffs(stop) - 1);
}

// The group's candidate list: lane b < 27 finds bucket b's range, and the
// sorted positions of the buckets' first min(count, 32) entries go to cidx in
// bucket order. Returns their number (at most 864). All lanes take part.
__device__ __forceinline__ uint32_t coop_candidates(const uint2* __restrict__ bucket, uint32_t cx, uint32_t cy,
                                                    uint32_t cz, uint32_t cell_mask, uint32_t base, uint32_t lane,
                                                    uint32_t* cidx) {
    uint32_t start = 0;
    uint32_t count = 0;
    if (lane < 27u) {
        const uint2 r = neighbour_range(bucket, cx, cy, cz, lane, cell_mask, base);
        start = r.x;
        count = r.y - r.x;
    }
    uint32_t inclusive = count;
#pragma unroll
    for (uint32_t o = 1; o < 32u; o <<= 1) {
        const uint32_t v = __shfl_up_sync(kFullMask, inclusive, o);
        if (lane >= o) {
            inclusive += v;
        }
    }
    const uint32_t total = __shfl_sync(kFullMask, inclusive, 31);
    const uint32_t offset = inclusive - count;
    for (uint32_t k = 0; k < count; ++k) {
        cidx[offset + k] = start + k;
    }
    __syncwarp();
    return total;
}

template <bool kCount>
__global__ void __launch_bounds__(kCoopWarps * 32) density_coop_kernel(const float4* __restrict__ spos,
                                                                       float4* __restrict__ svel,
                                                                       float4* __restrict__ spos2,
                                                                       const uint2* __restrict__ bucket,
                                                                       const TankConst* __restrict__ tanks,
                                                                       const uint16_t* __restrict__ stank, uint32_t n,
                                                                       const uint32_t* __restrict__ order,
                                                                       uint32_t* __restrict__ masks,
                                                                       StepCounters* __restrict__ counters,
                                                                       int all_tanks) {
    __shared__ uint32_t s_cidx[kCoopWarps][kCoopMaxCandidates];
    __shared__ float4 s_self[kCoopWarps][32];
    // Row i: the terms of the group's i-th particle against the 32 candidates
    // of a chunk (36 floats a row: conflict-free 16-byte reads of a column).
    __shared__ __align__(16) float s_term[kCoopWarps][32][36];
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t w = threadIdx.x >> 5;
    const uint32_t slot = (blockIdx.x * kCoopWarps + w) * 32u + lane;
    uint32_t p = slot;
    if (order != nullptr && p < n) {
        p = order[p];
    }
    bool valid = p < n;
    const uint32_t tank = valid && stank != nullptr ? stank[p] : 0u;
    const TankConst* t = tanks + tank;
    // A tank that sits this substep out is not integrated, and tanks never
    // share pairs, so its densities are not needed (pair counting visits all).
    if (!kCount && all_tanks == 0 && valid && __ldg(&t->active) == 0) {
        valid = false;
    }
    float4 self = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    uint32_t cx = 0;
    uint32_t cy = 0;
    uint32_t cz = 0;
    if (valid) {
        self = spos[p];
        const float h = __ldg(&t->h);
        cx = static_cast<uint32_t>(cell_coord(self.x, h));
        cy = static_cast<uint32_t>(cell_coord(self.y, h));
        cz = static_cast<uint32_t>(cell_coord(self.z, h));
    }
    s_self[w][lane] = self;
    uint32_t valid_mask = 0;
    uint32_t starts = coop_group_starts(valid, tank, cx, cy, cz, lane, valid_mask);
    float density = 0.0f;
    unsigned long long candidates = 0;
    unsigned long long in_range = 0;
    const float far = __int_as_float(0x7F800000);  // +inf: a padding lane's candidate
    while (starts != 0) {
        const uint32_t s = static_cast<uint32_t>(__ffs(starts) - 1);
        starts &= starts - 1u;
        const uint32_t e = coop_group_end(s, starts, valid_mask);
        const uint32_t m = e - s;
        const bool mine = lane >= s && lane < e;
        const TankConst* g = tanks + __shfl_sync(kFullMask, tank, s);
        const uint32_t gx = __shfl_sync(kFullMask, cx, s);
        const uint32_t gy = __shfl_sync(kFullMask, cy, s);
        const uint32_t gz = __shfl_sync(kFullMask, cz, s);
        const float h2 = __ldg(&g->h2);
        const float c6 = __ldg(&g->c_poly6);
        const float mass = __ldg(&g->mass);
        const float r2_far = __ldg(&g->r2_far);
        const float r2_near = __ldg(&g->r2_near);
        const uint32_t count = coop_candidates(bucket, gx, gy, gz, __ldg(&g->cell_mask), __ldg(&g->bucket_base),
                                               lane, s_cidx[w]);
        // max.NaN(term, +0) drops out-of-range terms while mass * c_poly6 > 0
        // (out of range d <= 0, so the term is negative or +0); otherwise the
        // reference's compare and select.
        const bool by_max = mass > 0.0f && c6 > 0.0f;
        const uint32_t chunks = (count + 31u) / 32u;
        for (uint32_t c = 0; c < chunks; ++c) {
            const uint32_t q = c * 32u + lane;
            const uint32_t left = count - c * 32u;
            const uint32_t live = left >= 32u ? kFullMask : ((1u << left) - 1u);
            float ox = far;
            float oy = far;
            float oz = far;
            if (q < count) {
                const float4 o = __ldg(&spos[s_cidx[w][q]]);
                ox = o.x;
                oy = o.y;
                oz = o.z;
            }
            uint32_t word = 0;
            for (uint32_t i = 0; i < m; ++i) {
                const float4 si = s_self[w][s + i];
                const float r2 = dot3(__fsub_rn(si.x, ox), __fsub_rn(si.y, oy), __fsub_rn(si.z, oz));
                // mass * poly6 (fluid_sph.cpp:24-31, :214).
                const float d = __fsub_rn(h2, r2);
                const float term = __fmul_rn(mass, __fmul_rn(__fmul_rn(__fmul_rn(c6, d), d), d));
                float kept;
                if (by_max) {
                    asm("max.NaN.f32 %0, %1, %2;" : "=f"(kept) : "f"(term), "f"(0.0f));
                } else {
                    kept = r2 >= h2 ? 0.0f : term;
                }
                s_term[w][i][lane] = kept;
                // Integrate skips distance >= h or <= 1e-6 (fluid_sph.cpp:245-248);
                // the particle itself (r2 = 0) fails the second test.
                const uint32_t used = __ballot_sync(kFullMask, !(r2 >= r2_far || r2 <= r2_near)) & live;
                if (lane == s + i) {
                    word = used;
                }
                if (kCount) {
                    const uint32_t near = __ballot_sync(kFullMask, r2 < h2) & live;
                    if (lane == 0) {
                        in_range += static_cast<unsigned long long>(__popc(near));
                    }
                }
            }
            __syncwarp();
            if (mine) {
                const float* row = s_term[w][lane - s];
#pragma unroll
                for (uint32_t k = 0; k < 32u; k += 4u) {
                    const float4 v = *reinterpret_cast<const float4*>(row + k);
                    density = __fadd_rn(density, v.x);
                    density = __fadd_rn(density, v.y);
                    density = __fadd_rn(density, v.z);
                    density = __fadd_rn(density, v.w);
                }
                masks[static_cast<size_t>(c) * n + slot] = word;
            }
            __syncwarp();
        }
        if (kCount && mine) {
            candidates += count;
        }
    }
    if (kCount) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            candidates += __shfl_down_sync(kFullMask, candidates, o);
        }
        if (lane == 0) {
            atomicAdd(&counters->candidates, candidates);
            atomicAdd(&counters->in_range, in_range);
        }
    }
    if (!valid) {
        return;
    }
    density = max_like_std(density, 1e-6f);
    const float pressure =
        max_like_std(__fmul_rn(__ldg(&t->stiffness), __fsub_rn(density, __ldg(&t->rest_density))), 0.0f);
    spos2[p] = make_float4(self.x, self.y, self.z, density);
    reinterpret_cast<float*>(svel)[4 * static_cast<size_t>(p) + 3] = pressure;
}

// Pressure and viscosity terms of one in-range pair with the two shared
// reciprocals: the operations of add_pair_force_rcp, whose sums add pv.xyz
// then pv.w / vyz in this order per axis.
__device__ __forceinline__ void pair_terms(const PairConst& k, const float4& self, const float4& sv,
                                           const float4& other, const float4& ov, float4& pv, float2& vyz) {
    const float ex = __fsub_rn(self.x, other.x);
    const float ey = __fsub_rn(self.y, other.y);
    const float ez = __fsub_rn(self.z, other.z);
    const float distance = __fsqrt_rn(dot3(ex, ey, ez));
    const float inv_distance = __frcp_rn(distance);
    const float other_density = max_like_std(other.w, 1e-6f);
    const float inv_density = __frcp_rn(other_density);
    const float ps = div_by(__fmul_rn(k.neg_mass, __fadd_rn(sv.w, ov.w)), __fmul_rn(2.0f, other_density),
                            __fmul_rn(0.5f, inv_density));
    const float d = __fsub_rn(k.h, distance);
    const float gs = __fmul_rn(__fmul_rn(k.c_spiky, d), d);
    pv.x = __fmul_rn(ps, __fmul_rn(gs, div_by(ex, distance, inv_distance)));
    pv.y = __fmul_rn(ps, __fmul_rn(gs, div_by(ey, distance, inv_distance)));
    pv.z = __fmul_rn(ps, __fmul_rn(gs, div_by(ez, distance, inv_distance)));
    const float lap = __fmul_rn(k.c_visc, d);
    pv.w = __fmul_rn(div_by(__fmul_rn(k.visc_mass, __fsub_rn(ov.x, sv.x)), other_density, inv_density), lap);
    vyz.x = __fmul_rn(div_by(__fmul_rn(k.visc_mass, __fsub_rn(ov.y, sv.y)), other_density, inv_density), lap);
    vyz.y = __fmul_rn(div_by(__fmul_rn(k.visc_mass, __fsub_rn(ov.z, sv.z)), other_density, inv_density), lap);
}

template <int kMinBlocks>
__global__ void __launch_bounds__(kCoopWarps * 32, kMinBlocks) integrate_coop_kernel(
    const float4* __restrict__ spos2, const float4* __restrict__ svel, const uint32_t* __restrict__ sorted_ids,
    const uint2* __restrict__ bucket, const TankConst* __restrict__ tanks, const uint16_t* __restrict__ stank,
    uint32_t n, const uint32_t* __restrict__ order, const uint32_t* __restrict__ masks, float4* __restrict__ pos_out,
    float4* __restrict__ vel_out) {
    __shared__ uint32_t s_cidx[kCoopWarps][kCoopMaxCandidates];
    __shared__ float4 s_selfp[kCoopWarps][32];
    __shared__ float4 s_selfv[kCoopWarps][32];
    __shared__ float4 s_pv[kCoopWarps][kCoopPairs];   // pressure xyz, viscosity x
    __shared__ float2 s_vyz[kCoopWarps][kCoopPairs];  // viscosity y, z
    __shared__ uint16_t s_pq[kCoopWarps][kCoopPairs];  // candidate of each listed pair
    __shared__ uint8_t s_pi[kCoopWarps][kCoopPairs];   // its particle, within the group
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t w = threadIdx.x >> 5;
    const uint32_t slot = (blockIdx.x * kCoopWarps + w) * 32u + lane;
    uint32_t p = slot;
    if (order != nullptr && p < n) {
        p = order[p];
    }
    bool valid = p < n;
    const uint32_t tank = valid && stank != nullptr ? stank[p] : 0u;
    const TankConst* t = tanks + tank;
    valid = valid && __ldg(&t->active) != 0;
    float4 self = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    float4 sv = self;
    uint32_t cx = 0;
    uint32_t cy = 0;
    uint32_t cz = 0;
    if (valid) {
        self = spos2[p];
        sv = svel[p];
        const float h = __ldg(&t->h);
        cx = static_cast<uint32_t>(cell_coord(self.x, h));
        cy = static_cast<uint32_t>(cell_coord(self.y, h));
        cz = static_cast<uint32_t>(cell_coord(self.z, h));
    }
    s_selfp[w][lane] = self;
    s_selfv[w][lane] = sv;
    uint32_t valid_mask = 0;
    uint32_t starts = coop_group_starts(valid, tank, cx, cy, cz, lane, valid_mask);
    float fx = 0.0f;
    float fy = 0.0f;
    float fz = 0.0f;
    while (starts != 0) {
        const uint32_t s = static_cast<uint32_t>(__ffs(starts) - 1);
        starts &= starts - 1u;
        const uint32_t e = coop_group_end(s, starts, valid_mask);
        const uint32_t m = e - s;
        const bool mine = lane >= s && lane < e;
        const TankConst* g = tanks + __shfl_sync(kFullMask, tank, s);
        PairConst k;
        k.h = __ldg(&g->h);
        k.c_spiky = __ldg(&g->c_spiky);
        k.c_visc = __ldg(&g->c_visc);
        k.neg_mass = __ldg(&g->neg_mass);
        k.visc_mass = __ldg(&g->visc_mass);
        const uint32_t count =
            coop_candidates(bucket, __shfl_sync(kFullMask, cx, s), __shfl_sync(kFullMask, cy, s),
                            __shfl_sync(kFullMask, cz, s), __ldg(&g->cell_mask), __ldg(&g->bucket_base), lane, s_cidx[w]);
        const uint32_t chunks = (count + 31u) / 32u;
        // This lane's particle: its pairs left to list and its place in the
        // mask words (chunk c, the bits not yet listed).
        uint32_t left = 0;
        uint32_t c = 0;
        uint32_t word = 0;
        if (mine) {
            for (uint32_t j = 0; j < chunks; ++j) {
                left += static_cast<uint32_t>(__popc(__ldg(&masks[static_cast<size_t>(j) * n + slot])));
            }
            if (chunks != 0) {
                word = __ldg(&masks[slot]);
            }
        }
        // Lanes a, a + 32, a + 64 own the sums of (particle a / 3, axis a % 3).
        float acc[3] = {0.0f, 0.0f, 0.0f};
        const uint32_t per_particle = kCoopPairs / m;
        while (__any_sync(kFullMask, left != 0)) {
            // List each particle's next pairs, in candidate order.
            const uint32_t take = min(left, per_particle);
            uint32_t first = take;
#pragma unroll
            for (uint32_t o = 1; o < 32u; o <<= 1) {
                const uint32_t v = __shfl_up_sync(kFullMask, first, o);
                if (lane >= o) {
                    first += v;
                }
            }
            const uint32_t total = __shfl_sync(kFullMask, first, 31);
            first -= take;
            for (uint32_t j = 0; j < take; ++j) {
                while (word == 0) {
                    ++c;
                    word = __ldg(&masks[static_cast<size_t>(c) * n + slot]);
                }
                const uint32_t bit = static_cast<uint32_t>(__ffs(word) - 1);
                word &= word - 1u;
                s_pq[w][first + j] = static_cast<uint16_t>(c * 32u + bit);
                s_pi[w][first + j] = static_cast<uint8_t>(lane - s);
            }
            left -= take;
            __syncwarp();
            // Pair terms, one pair per lane.
            for (uint32_t f = lane; f < total; f += 32u) {
                const uint32_t i = s + s_pi[w][f];
                const uint32_t q = s_cidx[w][s_pq[w][f]];
                float4 pv;
                float2 vyz;
                pair_terms(k, s_selfp[w][i], s_selfv[w][i], __ldg(&spos2[q]), __ldg(&svel[q]), pv, vyz);
                s_pv[w][f] = pv;
                s_vyz[w][f] = vyz;
            }
            __syncwarp();
            // Sums per (particle, axis): pressure then viscosity term of each
            // pair, pairs in order (fluid_sph.cpp:249-254).
#pragma unroll
            for (uint32_t r = 0; r < 3u; ++r) {
                const uint32_t a = lane + 32u * r;
                const uint32_t i = a / 3u;
                const uint32_t axis = a - 3u * i;
                const uint32_t src = min(s + i, 31u);
                const uint32_t from = __shfl_sync(kFullMask, first, src);
                const uint32_t n_i = __shfl_sync(kFullMask, take, src);
                if (i < m) {
                    for (uint32_t f = from; f < from + n_i; ++f) {
                        const float* pvf = reinterpret_cast<const float*>(&s_pv[w][f]);
                        const float vis = axis == 0u ? pvf[3] : reinterpret_cast<const float*>(&s_vyz[w][f])[axis - 1u];
                        acc[r] = __fadd_rn(__fadd_rn(acc[r], pvf[axis]), vis);
                    }
                }
            }
            __syncwarp();
        }
        // Hand each particle's three sums to its own lane.
        float* sums = reinterpret_cast<float*>(s_pv[w]);
#pragma unroll
        for (uint32_t r = 0; r < 3u; ++r) {
            const uint32_t a = lane + 32u * r;
            if (a < 3u * m) {
                sums[a] = acc[r];
            }
        }
        __syncwarp();
        if (mine) {
            const uint32_t i = lane - s;
            fx = sums[3u * i];
            fy = sums[3u * i + 1u];
            fz = sums[3u * i + 2u];
        }
        __syncwarp();
    }
    if (!valid) {
        return;
    }
    finish_particle(t, self, max_like_std(self.w, 1e-6f), sv.x, sv.y, sv.z, sv.w, fx, fy, fz, sorted_ids[p], pos_out,
                    vel_out);
}

// ---- learned coarse step ------------------------------------------------------
//
// The learned step splits integrate in two: `features_kernel` computes the
// plain SPH force of each particle exactly as integrate_mask_kernel does and,
// over the same pairs, the 32 features the correction MLP reads; the MLP
// turns features into an acceleration correction; `finish_learned_kernel`
// adds it to the plain acceleration and advances the particle exactly as the
// plain integrate does. With a zero correction the result is bit-identical to
// the plain substep.
//
// Features of particle i (h the kernel radius, D the substep, rho0 and k the
// rest density and stiffness; sums over the in-range pairs j, u = (x_j -
// x_i) / h, w = (1 - |u|)^2):
//   0  (rho_i - rho0) / rho0          1  p_i / (k rho0)
//   2-4  v_i D / h                    5-7  (F_i / rho_i) D^2 / h
//   8  pairs / 32                     9  sum w
//   10-12  sum w u                    13-15  sum w (v_j - v_i) D / h
//   16-21  sum w u_a u_b (xx yy zz xy xz yz)
//   22-24  sum w (p_j - p_i) / (k rho0) u
//   25  sum w (rho_j - rho_i) / rho0
//   26-28  min(max((x_i - wall_low) / h, 0), 4)   29-31  same for the high walls
constexpr int kFeatures = 32;

template <int kBlock, int kList, int kMinBlocks = 1>
__global__ void __launch_bounds__(kBlock, kMinBlocks) features_kernel(const float4* __restrict__ spos2,
                                                          const float4* __restrict__ svel,
                                                          const uint32_t* __restrict__ sorted_ids,
                                                          const uint2* __restrict__ bucket,
                                                          const TankConst* __restrict__ tanks,
                                                          const uint16_t* __restrict__ stank, uint32_t n,
                                                          const uint32_t* __restrict__ order,
                                                          const uint32_t* __restrict__ masks,
                                                          float4* __restrict__ force_out,
                                                          float* __restrict__ features_out, int id_order,
                                                          const float* __restrict__ norm_mean,
                                                          const float* __restrict__ norm_inv_std,
                                                          uint8_t* __restrict__ x_tiles) {
    static_assert(kList >= 32, "a pair list must hold a whole bucket");
    // The MLP launched after this pass may set up (weights, tensor memory)
    // once every block of this one has started; it waits for this grid's
    // end before it reads a tile.
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    __shared__ uint32_t list[kList][kBlock];
    const uint32_t slot = blockIdx.x * kBlock + threadIdx.x;
    uint32_t p = slot;
    if (order != nullptr && p < n) {
        p = order[p];
    }
    // Features of a tank that sits this substep out are not used (its finish
    // is skipped), so its particles leave the walk.
    bool valid = p < n;
    const TankConst* t = tanks + (valid && stank != nullptr ? stank[p] : 0);
    valid = valid && (id_order != 0 || __ldg(&t->active) != 0);
    const uint32_t live = __ballot_sync(0xFFFFFFFFu, valid);
    if (!valid) {
        return;
    }
    PairConst k;
    k.h = __ldg(&t->h);
    k.c_spiky = __ldg(&t->c_spiky);
    k.c_visc = __ldg(&t->c_visc);
    k.neg_mass = __ldg(&t->neg_mass);
    k.visc_mass = __ldg(&t->visc_mass);
    const uint32_t cell_mask = __ldg(&t->cell_mask);
    const uint32_t base = __ldg(&t->bucket_base);
    const float4 self = spos2[p];
    const float4 sv = svel[p];
    const uint32_t cx = static_cast<uint32_t>(cell_coord(self.x, k.h));
    const uint32_t cy = static_cast<uint32_t>(cell_coord(self.y, k.h));
    const uint32_t cz = static_cast<uint32_t>(cell_coord(self.z, k.h));
    const float rho0 = __ldg(&t->rest_density);
    const float stiff = __ldg(&t->stiffness);
    const float dt = __ldg(&t->dt);
    const float inv_h = 1.0f / k.h;
    const float vscale = dt * inv_h;
    const float inv_prho = 1.0f / (stiff * rho0);
    float fx = 0.0f;
    float fy = 0.0f;
    float fz = 0.0f;
    float f[kFeatures];
#pragma unroll
    for (int q = 0; q < kFeatures; ++q) {
        f[q] = 0.0f;
    }
    uint32_t pairs = 0;
    // The feature sums reuse the pair force's offset, distance and velocity
    // difference (u = -e / h, |u| = distance / h) and leave the constant
    // factors (D / h, 1 / (k rho0), 1 / rho0) to the end; the features are
    // MLP inputs, rounded to BF16, so their sums use FMA.
    const float neg_inv_h = -inv_h;
    auto visit = [&](uint32_t q) {
        float4 other = __ldg(&spos2[q]);
        float4 ov = __ldg(&svel[q]);
        PairParts e;
        add_pair_force_rcp(k, self, sv.x, sv.y, sv.z, sv.w, other, ov, fx, fy, fz, e);
        const float ux = e.ex * neg_inv_h;
        const float uy = e.ey * neg_inv_h;
        const float uz = e.ez * neg_inv_h;
        const float om = 1.0f - e.distance * inv_h;
        const float w = om * om;
        const float wx = w * ux;
        const float wy = w * uy;
        const float wz = w * uz;
        f[9] += w;
        f[10] += wx;
        f[11] += wy;
        f[12] += wz;
        f[13] = fmaf(w, e.dvx, f[13]);
        f[14] = fmaf(w, e.dvy, f[14]);
        f[15] = fmaf(w, e.dvz, f[15]);
        f[16] = fmaf(wx, ux, f[16]);
        f[17] = fmaf(wy, uy, f[17]);
        f[18] = fmaf(wz, uz, f[18]);
        f[19] = fmaf(wx, uy, f[19]);
        f[20] = fmaf(wx, uz, f[20]);
        f[21] = fmaf(wy, uz, f[21]);
        const float wdp = w * (ov.w - sv.w);
        f[22] = fmaf(wdp, ux, f[22]);
        f[23] = fmaf(wdp, uy, f[23]);
        f[24] = fmaf(wdp, uz, f[24]);
        f[25] = fmaf(w, other.w - self.w, f[25]);
        ++pairs;
    };
    uint32_t listed = 0;
    // Three buckets at a time: their mask words, then the first slots of the
    // buckets with pairs, loaded back to back (as integrate_mask_kernel).
    constexpr uint32_t kGroup = 3;
    for (uint32_t b0 = 0; b0 < 27u; b0 += kGroup) {
        uint32_t words[kGroup];
        uint32_t firsts[kGroup];
#pragma unroll
        for (uint32_t j = 0; j < kGroup; ++j) {
            words[j] = __ldg(&masks[static_cast<size_t>(b0 + j) * n + slot]);
        }
#pragma unroll
        for (uint32_t j = 0; j < kGroup; ++j) {
            firsts[j] = words[j] != 0 ? neighbour_range(bucket, cx, cy, cz, b0 + j, cell_mask, base).x : 0u;
        }
#pragma unroll
        for (uint32_t j = 0; j < kGroup; ++j) {
            uint32_t word = words[j];
            // Every lane drains together when any lane's list is about to overflow.
            if (__any_sync(live, listed + static_cast<uint32_t>(__popc(word)) > static_cast<uint32_t>(kList))) {
                for (uint32_t e = 0; e < listed; ++e) {
                    visit(list[e][threadIdx.x]);
                }
                listed = 0;
            }
            while (word != 0) {
                uint32_t s = static_cast<uint32_t>(__ffs(word) - 1);
                word &= word - 1;
                list[listed][threadIdx.x] = firsts[j] + s;
                ++listed;
            }
        }
    }
    for (uint32_t e = 0; e < listed; ++e) {
        visit(list[e][threadIdx.x]);
    }
#pragma unroll
    for (int q = 13; q < 16; ++q) {
        f[q] *= vscale;
    }
#pragma unroll
    for (int q = 22; q < 25; ++q) {
        f[q] *= inv_prho;
    }
    f[25] /= rho0;
    const float density = max_like_std(self.w, 1e-6f);
    f[0] = (self.w - rho0) / rho0;
    f[1] = sv.w * inv_prho;
    f[2] = sv.x * vscale;
    f[3] = sv.y * vscale;
    f[4] = sv.z * vscale;
    f[5] = fx / density * dt * vscale;
    f[6] = fy / density * dt * vscale;
    f[7] = fz / density * dt * vscale;
    f[8] = pairs * (1.0f / 32.0f);
    const float pos[3] = {self.x, self.y, self.z};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        f[26 + a] = fminf(fmaxf((pos[a] - __ldg(&t->low[a])) * inv_h, 0.0f), 4.0f);
        f[29 + a] = fminf(fmaxf((__ldg(&t->high[a]) - pos[a]) * inv_h, 0.0f), 4.0f);
    }
    force_out[p] = make_float4(fx, fy, fz, 0.0f);
    if (x_tiles != nullptr) {
        // The MLP's input row p: (f - mean) / std rounded to BF16, as the
        // forward pass would convert it, in its tile layout.
        uint8_t* tile = x_tiles + static_cast<size_t>(p / mlp::kTile) * mlp::kXTileBytes;
        const uint32_t local = p % mlp::kTile;
#pragma unroll
        for (uint32_t c = 0; c < kFeatures / 8; ++c) {
            uint32_t word[4];
#pragma unroll
            for (uint32_t k = 0; k < 4; ++k) {
                const uint32_t a = 8 * c + 2 * k;
                const float v0 = (f[a] - __ldg(&norm_mean[a])) * __ldg(&norm_inv_std[a]);
                const float v1 = (f[a + 1] - __ldg(&norm_mean[a + 1])) * __ldg(&norm_inv_std[a + 1]);
                const __nv_bfloat162 pair = __floats2bfloat162_rn(v0, v1);
                word[k] = *reinterpret_cast<const uint32_t*>(&pair);
            }
            *reinterpret_cast<uint4*>(tile + mlp::x_tile_offset(local, c)) = make_uint4(word[0], word[1], word[2], word[3]);
        }
    } else if (features_out != nullptr) {
        uint32_t row = id_order ? sorted_ids[p] : p;
        float4* dst = reinterpret_cast<float4*>(features_out + static_cast<size_t>(row) * kFeatures);
#pragma unroll
        for (int q = 0; q < kFeatures / 4; ++q) {
            dst[q] = make_float4(f[4 * q], f[4 * q + 1], f[4 * q + 2], f[4 * q + 3]);
        }
    }
}

// The correction's net force on each tank, as the sum of its particles'
// corrections in 2^-24 m/s^2 fixed point: integer sums do not depend on the
// order of the atomics, so the mean (and the step) is the same on every run.
// sums holds kCorrectionSumWords per tank: x, y, z and the particle count.
constexpr float kCorrectionFixed = 16777216.0f;  // 2^24
constexpr float kCorrectionFixedMax = 1.0e9f;    // |correction| beyond this (or NaN) counts as 0
__device__ __forceinline__ long long correction_fixed(float v) {
    return fabsf(v) <= kCorrectionFixedMax ? __float2ll_rn(v * kCorrectionFixed) : 0ll;
}

// Block b takes a contiguous range of sorted positions (tanks are contiguous
// in the sorted order): each lane adds its particles' fixed-point corrections
// into 64-bit registers, and the warp reduces them and adds them to the
// tank's sums when its tank changes and at the end. Integer sums: the result
// does not depend on how the work is split.
__global__ void __launch_bounds__(256) correction_sums_kernel(const float4* __restrict__ correction,
                                                              const TankConst* __restrict__ tanks,
                                                              const uint16_t* __restrict__ stank, uint32_t n,
                                                              unsigned long long* __restrict__ sums) {
    // Launched programmatically after the MLP: wait for its corrections.
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    asm volatile("griddepcontrol.wait;" ::: "memory");
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t warp = threadIdx.x >> 5;
    const size_t per_block = ((static_cast<size_t>(n) + gridDim.x - 1) / gridDim.x + 31) & ~static_cast<size_t>(31);
    const size_t begin = blockIdx.x * per_block;
    const size_t end = begin + per_block < n ? begin + per_block : n;
    long long x = 0;
    long long y = 0;
    long long z = 0;
    unsigned long long count = 0;
    uint32_t current = 0xFFFFFFFFu;  // the tank the lanes' sums belong to (warp-uniform)
    auto flush = [&]() {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            x += __shfl_down_sync(0xFFFFFFFFu, x, o);
            y += __shfl_down_sync(0xFFFFFFFFu, y, o);
            z += __shfl_down_sync(0xFFFFFFFFu, z, o);
            count += __shfl_down_sync(0xFFFFFFFFu, count, o);
        }
        if (lane == 0 && current != 0xFFFFFFFFu && count != 0) {
            unsigned long long* s = sums + static_cast<size_t>(current) * kCorrectionSumWords;
            atomicAdd(&s[0], static_cast<unsigned long long>(x));
            atomicAdd(&s[1], static_cast<unsigned long long>(y));
            atomicAdd(&s[2], static_cast<unsigned long long>(z));
            atomicAdd(&s[3], count);
        }
        x = 0;
        y = 0;
        z = 0;
        count = 0;
    };
    for (size_t first = begin + 32u * warp; first < end; first += blockDim.x) {
        const size_t p = first + lane;
        const bool valid = p < end;
        const uint32_t t = valid && stank != nullptr ? stank[p] : 0u;
        const bool counted = valid && __ldg(&tanks[t].active) != 0;
        const uint32_t key = counted ? t : 0xFFFFFFFFu;
        const uint32_t lead = __shfl_sync(0xFFFFFFFFu, key, 0);
        long long cx = 0;
        long long cy = 0;
        long long cz = 0;
        if (counted) {
            const float4 c = correction[p];
            cx = correction_fixed(c.x);
            cy = correction_fixed(c.y);
            cz = correction_fixed(c.z);
        }
        if (__all_sync(0xFFFFFFFFu, key == lead) && lead != 0xFFFFFFFFu) {
            if (lead != current) {
                flush();
                current = lead;
            }
            x += cx;
            y += cy;
            z += cz;
            count += 1;
        } else if (counted) {
            // Lanes of several tanks (or uncounted lanes): add now.
            unsigned long long* s = sums + static_cast<size_t>(t) * kCorrectionSumWords;
            atomicAdd(&s[0], static_cast<unsigned long long>(cx));
            atomicAdd(&s[1], static_cast<unsigned long long>(cy));
            atomicAdd(&s[2], static_cast<unsigned long long>(cz));
            atomicAdd(&s[3], 1ull);
        }
    }
    flush();
}

__global__ void __launch_bounds__(256) finish_learned_kernel(const float4* __restrict__ spos2,
                                                             const float4* __restrict__ svel,
                                                             const uint32_t* __restrict__ sorted_ids,
                                                             const TankConst* __restrict__ tanks,
                                                             const uint16_t* __restrict__ stank, uint32_t n,
                                                             const float4* __restrict__ force,
                                                             const float4* __restrict__ correction,
                                                             const unsigned long long* __restrict__ sums,
                                                             uint32_t free_axes, float4* __restrict__ pos_out,
                                                             float4* __restrict__ vel_out) {
    // Launched programmatically after the MLP or the sums: wait for them.
    asm volatile("griddepcontrol.wait;" ::: "memory");
    uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) {
        return;
    }
    const uint32_t tank = stank != nullptr ? stank[p] : 0u;
    const TankConst* t = tanks + tank;
    if (__ldg(&t->active) == 0) {
        return;
    }
    const float4 self = spos2[p];
    const float4 sv = svel[p];
    const float4 fo = force[p];
    float4 da = correction != nullptr ? correction[p] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (correction != nullptr && sums != nullptr) {
        // No net force along the chosen axes: the tank's mean correction is
        // taken off every particle.
        const unsigned long long* s = sums + static_cast<size_t>(tank) * kCorrectionSumWords;
        const double scale = 1.0 / (static_cast<double>(kCorrectionFixed) * static_cast<double>(__ldg(&s[3])));
        if (free_axes & 1u) {
            da.x -= static_cast<float>(static_cast<double>(static_cast<long long>(__ldg(&s[0]))) * scale);
        }
        if (free_axes & 2u) {
            da.y -= static_cast<float>(static_cast<double>(static_cast<long long>(__ldg(&s[1]))) * scale);
        }
        if (free_axes & 4u) {
            da.z -= static_cast<float>(static_cast<double>(static_cast<long long>(__ldg(&s[2]))) * scale);
        }
    }
    finish_particle(t, self, max_like_std(self.w, 1e-6f), sv.x, sv.y, sv.z, sv.w, fo.x, fo.y, fo.z, sorted_ids[p],
                    pos_out, vel_out, da);
}

// Division self-test: counts x / y where the reciprocal-based quotient and
// IEEE division differ in value (signed zeros compare equal).
__global__ void division_selftest_kernel(uint64_t seed, uint64_t count, int mode, unsigned long long* mismatches) {
    uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
    unsigned long long bad = 0;
    for (uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < count; i += stride) {
        float x;
        float y;
        if (mode == 6) {
            // Consecutive floats x from the one with the seed's high 32 bits,
            // y the float with its low 32 bits: the quotients x / y in [0, 1)
            // of the surface field's d2 / radius^2.
            x = __uint_as_float(static_cast<uint32_t>(seed >> 32) + static_cast<uint32_t>(i));
            y = __uint_as_float(static_cast<uint32_t>(seed));
        } else if (mode == 0) {
            // Every divisor mantissa in [1, 2) against dividends from a mixer.
            uint32_t ym = static_cast<uint32_t>(i & 0x7FFFFFu);
            uint64_t z = (i >> 23) * 0x9E3779B97F4A7C15ULL + seed;
            z = (z ^ (z >> 31)) * 0xBF58476D1CE4E5B9ULL;
            uint32_t xb = 0x3F800000u | static_cast<uint32_t>((z >> 20) & 0x7FFFFFu);
            x = __uint_as_float(xb);
            y = __uint_as_float(0x3F800000u | ym);
        } else {
            // Random signs, mantissas and exponents over 2^-60 .. 2^60.
            uint64_t z = i * 0x9E3779B97F4A7C15ULL + seed;
            z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
            z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
            z ^= z >> 31;
            uint32_t ex = 67u + static_cast<uint32_t>((z >> 8) % 121u);
            uint32_t ey = 67u + static_cast<uint32_t>((z >> 16) % 121u);
            x = __uint_as_float((static_cast<uint32_t>(z >> 63) << 31) | (ex << 23) |
                                static_cast<uint32_t>((z >> 24) & 0x7FFFFFu));
            y = __uint_as_float((static_cast<uint32_t>((z >> 62) & 1u) << 31) | (ey << 23) |
                                static_cast<uint32_t>((z >> 40) & 0x7FFFFFu));
        }
        float want;
        float got;
        if (mode <= 1 || mode == 6) {
            want = __fdiv_rn(x, y);
            got = div_by(x, y, __frcp_rn(y));
        } else {
            // Packed f32x2 arithmetic against the scalar operations.
            float u = __fmul_rn(x, 0.75f);
            float v = __fadd_rn(y, 0.125f);
            unsigned long long px = pack2(x, u);
            unsigned long long py = pack2(y, v);
            float lo;
            float hi;
            if (mode == 2) {
                unpack2(mul2(px, py), lo, hi);
                want = __fmul_rn(x, y);
                got = lo;
                if (hi != __fmul_rn(u, v)) {
                    ++bad;
                }
            } else if (mode == 3) {
                unpack2(add2(px, py), lo, hi);
                want = __fadd_rn(x, y);
                got = lo;
                if (hi != __fadd_rn(u, v)) {
                    ++bad;
                }
            } else if (mode == 4) {
                unpack2(sub2(px, py), lo, hi);
                want = __fsub_rn(x, y);
                got = lo;
                if (hi != __fsub_rn(u, v)) {
                    ++bad;
                }
            } else {
                // The squared-distance chain (x*x + y*y) + u*u.
                unsigned long long pu = pack2(u, v);
                unpack2(add2(add2(mul2(px, px), mul2(py, py)), mul2(pu, pu)), lo, hi);
                want = __fadd_rn(__fadd_rn(__fmul_rn(x, x), __fmul_rn(y, y)), __fmul_rn(u, u));
                got = lo;
            }
        }
        if (want != got) {
            ++bad;
        }
    }
    if (bad != 0) {
        atomicAdd(mismatches, bad);
    }
}

}  // namespace

namespace {

// The staged integrate shapes: 128 threads with 1,248 data entries (55 KB of
// shared memory, four blocks an SM) or 256 threads with 2,016 (94 KB, two).
// The data areas hold a 99th-percentile block of the 1M dam break (973 and
// 1,419 entries on average, 1,245 and 1,842 at the 99th percentile).
#define SPH_STAGED_128 128u, 48u, 1248u, 9u, 4
#define SPH_STAGED_256 256u, 48u, 2016u, 10u, 2

template <uint32_t kThreads, uint32_t kList, uint32_t kCap, uint32_t kTableBits, int kMinBlocks>
constexpr size_t staged_bytes() {
    return staged::Layout<kThreads, kList, kCap, (1u << kTableBits)>::kBytes;
}

std::mutex g_staged_guard;
uint64_t g_staged_ready = 0;  // bit d: the attributes are set on device d

template <uint32_t kThreads, uint32_t kList, uint32_t kCap, uint32_t kTableBits, int kMinBlocks>
cudaError_t launch_staged(const float4* spos2, const float4* svel, const uint32_t* sorted_ids, const uint2* bucket,
                          const TankConst* tanks, const uint16_t* stank, uint32_t n, const uint32_t* order,
                          const uint32_t* masks, float4* pos, float4* vel, cudaStream_t stream) {
    constexpr size_t bytes = staged_bytes<kThreads, kList, kCap, kTableBits, kMinBlocks>();
    integrate_staged_kernel<kThreads, kList, kCap, kTableBits, kMinBlocks>
        <<<(n + kThreads - 1) / kThreads, kThreads, bytes, stream>>>(spos2, svel, sorted_ids, bucket, tanks, stank, n,
                                                                     order, masks, pos, vel);
    return cudaGetLastError();
}

}  // namespace

namespace {

__global__ void __launch_bounds__(256) scatter_rows_kernel(const float4* __restrict__ src,
                                                           const uint32_t* __restrict__ ids, uint32_t n,
                                                           float4* __restrict__ dst) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < n) {
        dst[ids[p]] = src[p];
    }
}

}  // namespace

cudaError_t launch_scatter_rows(const float4* src, const uint32_t* ids, uint32_t n, float4* dst, cudaStream_t stream) {
    if (n == 0) {
        return cudaSuccess;
    }
    scatter_rows_kernel<<<(n + 255) / 256, 256, 0, stream>>>(src, ids, n, dst);
    return cudaGetLastError();
}

cudaError_t prepare_staged_integrate() {
    int device = 0;
    cudaError_t e = cudaGetDevice(&device);
    if (e != cudaSuccess) {
        return e;
    }
    std::lock_guard<std::mutex> lock(g_staged_guard);
    if (device < 64 && (g_staged_ready >> device & 1u) != 0) {
        return cudaSuccess;
    }
    e = cudaFuncSetAttribute(integrate_staged_kernel<SPH_STAGED_128>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             static_cast<int>(staged_bytes<SPH_STAGED_128>()));
    if (e == cudaSuccess) {
        e = cudaFuncSetAttribute(integrate_staged_kernel<SPH_STAGED_256>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(staged_bytes<SPH_STAGED_256>()));
    }
    if (e == cudaSuccess && device < 64) {
        g_staged_ready |= 1ull << device;
    }
    return e;
}

cudaError_t launch_density(const float4* spos, float4* svel, float4* spos2, const uint2* bucket, const TankConst* tanks,
                           const uint16_t* stank, uint32_t n, StepCounters* counters, cudaStream_t stream,
                           const NeighbourTuning& tuning) {
    if (n == 0) {
        return cudaSuccess;
    }
    if (tuning.variant == 0) {
        uint32_t blocks = (n + 127) / 128;
        if (counters != nullptr) {
            density_kernel<true><<<blocks, 128, 0, stream>>>(spos, svel, spos2, bucket, tanks, stank, n, tuning.order, counters);
        } else {
            density_kernel<false><<<blocks, 128, 0, stream>>>(spos, svel, spos2, bucket, tanks, stank, n, tuning.order, nullptr);
        }
        return cudaGetLastError();
    }
    if (tuning.variant == 5) {
        const uint32_t blocks = (n + kCoopWarps * 32u - 1u) / (kCoopWarps * 32u);
        if (counters != nullptr) {
            density_coop_kernel<true><<<blocks, kCoopWarps * 32u, 0, stream>>>(spos, svel, spos2, bucket, tanks, stank, n,
                                                                             tuning.order, tuning.masks, counters, 1);
        } else {
            density_coop_kernel<false><<<blocks, kCoopWarps * 32u, 0, stream>>>(
                spos, svel, spos2, bucket, tanks, stank, n, tuning.order, tuning.masks, nullptr, tuning.all_tanks ? 1 : 0);
        }
        return cudaGetLastError();
    }
    if (tuning.variant == 4 || tuning.variant == 6) {
        uint32_t blocks = (n + 127) / 128;
        if (counters != nullptr) {
            density_mask_kernel<true><<<blocks, 128, 0, stream>>>(spos, svel, spos2, bucket, tanks, stank, n,
                                                                  tuning.order, tuning.masks, counters, 1);
        } else {
            density_mask_kernel<false><<<blocks, 128, 0, stream>>>(spos, svel, spos2, bucket, tanks, stank, n,
                                                                   tuning.order, tuning.masks, nullptr,
                                                                   tuning.all_tanks ? 1 : 0);
        }
        return cudaGetLastError();
    }
    if (tuning.variant >= 2) {
        uint32_t blocks = (n + 127) / 128;
        if (counters != nullptr) {
            density_list_kernel<true, false><<<blocks, 128, 0, stream>>>(spos, svel, spos2, bucket, tanks, stank, n,
                                                                  tuning.order, tuning.pair_list, tuning.pair_count, tuning.list_cap,
                                                                  counters);
        } else {
            density_list_kernel<false, false><<<blocks, 128, 0, stream>>>(spos, svel, spos2, bucket, tanks, stank, n,
                                                                   tuning.order, tuning.pair_list, tuning.pair_count,
                                                                   tuning.list_cap, nullptr);
        }
        return cudaGetLastError();
    }
    uint32_t threads = tuning.block;
    uint32_t blocks = (n + threads - 1) / threads;
    if (counters != nullptr) {
        density_flat_kernel<true><<<blocks, threads, 0, stream>>>(spos, svel, spos2, bucket, tanks, stank, n, tuning.order, counters);
    } else {
        density_flat_kernel<false><<<blocks, threads, 0, stream>>>(spos, svel, spos2, bucket, tanks, stank, n, tuning.order, nullptr);
    }
    return cudaGetLastError();
}

cudaError_t launch_integrate(const float4* spos2, const float4* svel, const uint32_t* sorted_ids, const uint2* bucket,
                             const TankConst* tanks, const uint16_t* stank, uint32_t n, float4* pos, float4* vel,
                             cudaStream_t stream, const NeighbourTuning& tuning) {
    if (n == 0) {
        return cudaSuccess;
    }
    const uint32_t slot_end = std::min(tuning.slot_end, n);
    if ((tuning.variant != 4 || tuning.order == nullptr) && (tuning.slot_begin != 0 || slot_end != n)) {
        return cudaErrorInvalidValue;  // a slot range needs the mask kernel and a processing order
    }
    if (tuning.slot_begin >= slot_end) {
        return cudaSuccess;
    }
    if (tuning.variant == 0) {
        integrate_kernel<<<(n + 127) / 128, 128, 0, stream>>>(spos2, svel, sorted_ids, bucket, tanks, stank, n, tuning.order, pos,
                                                              vel);
        return cudaGetLastError();
    }
    if (tuning.variant == 5) {
        const uint32_t blocks = (n + kCoopWarps * 32u - 1u) / (kCoopWarps * 32u);
        integrate_coop_kernel<1><<<blocks, kCoopWarps * 32u, 0, stream>>>(spos2, svel, sorted_ids, bucket, tanks, stank, n,
                                                                        tuning.order, tuning.masks, pos, vel);
        return cudaGetLastError();
    }
    if (tuning.variant == 6) {
        const cudaError_t prepared = prepare_staged_integrate();
        if (prepared != cudaSuccess) {
            return prepared;
        }
        if (tuning.block == 256) {
            return launch_staged<SPH_STAGED_256>(spos2, svel, sorted_ids, bucket, tanks, stank, n, tuning.order,
                                                 tuning.masks, pos, vel, stream);
        }
        return launch_staged<SPH_STAGED_128>(spos2, svel, sorted_ids, bucket, tanks, stank, n, tuning.order,
                                             tuning.masks, pos, vel, stream);
    }
    if (tuning.variant == 4) {
        const uint32_t b = tuning.slot_begin;
        const uint32_t slots = slot_end - b;
        const uint32_t* order = tuning.order != nullptr ? tuning.order + b : nullptr;
        const uint32_t* masks = tuning.masks + b;
        // programmatic: the launch may begin while the one before it in the
        // stream finishes (that launch must not write what this one reads).
        cudaLaunchAttribute attr{};
        attr.id = cudaLaunchAttributeProgrammaticStreamSerialization;
        attr.val.programmaticStreamSerializationAllowed = 1;
        auto launch = [&](auto kernel, uint32_t block) {
            cudaLaunchConfig_t cfg{};
            cfg.gridDim = dim3((slots + block - 1) / block);
            cfg.blockDim = dim3(block);
            cfg.stream = stream;
            cfg.attrs = tuning.programmatic ? &attr : nullptr;
            cfg.numAttrs = tuning.programmatic ? 1 : 0;
            return cudaLaunchKernelEx(&cfg, kernel, spos2, svel, sorted_ids, bucket, tanks, stank, n, order, masks,
                                      pos, vel, slots);
        };
        switch (tuning.block) {
        case 64:
            return launch(integrate_mask_kernel<64, 48>, 64);
        case 256:
            return launch(integrate_mask_kernel<256, 32>, 256);
        default:
            return launch(integrate_mask_kernel<128, 40, 9>, 128);
        }
    }
    if (tuning.variant >= 2) {
        bool rcp = tuning.variant == 3;
        switch (tuning.block) {
        case 64:
            if (rcp) {
                integrate_list_kernel<64, true><<<(n + 63) / 64, 64, 0, stream>>>(
                    spos2, svel, sorted_ids, bucket, tanks, stank, n, tuning.order, tuning.pair_list, tuning.pair_count,
                    tuning.list_cap, pos, vel);
            } else {
                integrate_list_kernel<64, false><<<(n + 63) / 64, 64, 0, stream>>>(
                    spos2, svel, sorted_ids, bucket, tanks, stank, n, tuning.order, tuning.pair_list, tuning.pair_count,
                    tuning.list_cap, pos, vel);
            }
            break;
        case 256:
            if (rcp) {
                integrate_list_kernel<256, true><<<(n + 255) / 256, 256, 0, stream>>>(
                    spos2, svel, sorted_ids, bucket, tanks, stank, n, tuning.order, tuning.pair_list, tuning.pair_count,
                    tuning.list_cap, pos, vel);
            } else {
                integrate_list_kernel<256, false><<<(n + 255) / 256, 256, 0, stream>>>(
                    spos2, svel, sorted_ids, bucket, tanks, stank, n, tuning.order, tuning.pair_list, tuning.pair_count,
                    tuning.list_cap, pos, vel);
            }
            break;
        default:
            if (rcp) {
                integrate_list_kernel<128, true><<<(n + 127) / 128, 128, 0, stream>>>(
                    spos2, svel, sorted_ids, bucket, tanks, stank, n, tuning.order, tuning.pair_list, tuning.pair_count,
                    tuning.list_cap, pos, vel);
            } else {
                integrate_list_kernel<128, false><<<(n + 127) / 128, 128, 0, stream>>>(
                    spos2, svel, sorted_ids, bucket, tanks, stank, n, tuning.order, tuning.pair_list, tuning.pair_count,
                    tuning.list_cap, pos, vel);
            }
            break;
        }
        return cudaGetLastError();
    }
    uint32_t threads = tuning.block;
    uint32_t blocks = (n + threads - 1) / threads;
    size_t smem = static_cast<size_t>(tuning.queue) * threads * sizeof(uint32_t);
    switch (tuning.queue) {
    case 8:
        integrate_queued_kernel<8><<<blocks, threads, smem, stream>>>(spos2, svel, sorted_ids, bucket, tanks, stank, n,
                                                                      tuning.order, pos, vel);
        break;
    case 16:
        integrate_queued_kernel<16><<<blocks, threads, smem, stream>>>(spos2, svel, sorted_ids, bucket, tanks, stank,
                                                                       n, tuning.order, pos, vel);
        break;
    case 32:
        integrate_queued_kernel<32><<<blocks, threads, smem, stream>>>(spos2, svel, sorted_ids, bucket, tanks, stank,
                                                                       n, tuning.order, pos, vel);
        break;
    default:
        integrate_queued_kernel<24><<<blocks, threads, smem, stream>>>(spos2, svel, sorted_ids, bucket, tanks, stank,
                                                                       n, tuning.order, pos, vel);
        break;
    }
    return cudaGetLastError();
}

cudaError_t launch_fields(const float4* pos, const uint16_t* tank_of, const TankConst* tanks, uint32_t n,
                          float4* out, cudaStream_t stream) {
    fields_kernel<<<(n + 255) / 256, 256, 0, stream>>>(pos, tank_of, tanks, n, out);
    return cudaGetLastError();
}

cudaError_t launch_colliders(float4* pos, float4* vel, const uint16_t* tank_of, const TankConst* tanks, uint32_t n,
                             cudaStream_t stream) {
    colliders_kernel<<<(n + 255) / 256, 256, 0, stream>>>(pos, vel, tank_of, tanks, n);
    return cudaGetLastError();
}

cudaError_t launch_emit(const TankConst* tank, uint32_t first, uint32_t count, float4* pos, float4* vel, float4* prev,
                        cudaStream_t stream) {
    if (count == 0) {
        return cudaSuccess;
    }
    emit_kernel<<<(count + 255) / 256, 256, 0, stream>>>(tank, first, count, pos, vel, prev);
    return cudaGetLastError();
}

cudaError_t launch_stats(const float4* pos, const float4* vel, const uint16_t* tank_of, const TankConst* tanks,
                         uint32_t n, double* acc, cudaStream_t stream) {
    if (n == 0) {
        return cudaSuccess;
    }
    int device = 0;
    int sms = 152;
    if (cudaGetDevice(&device) == cudaSuccess) {
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    }
    uint32_t blocks = (n + 255) / 256;
    blocks = std::min<uint32_t>(blocks, 4u * static_cast<uint32_t>(sms));
    stats_kernel<<<blocks, 256, 0, stream>>>(pos, vel, tank_of, tanks, n, acc);
    return cudaGetLastError();
}

cudaError_t launch_count_nonfinite(const float4* pos, const float4* vel, uint32_t n, uint32_t* out, cudaStream_t stream) {
    if (n == 0) {
        return cudaSuccess;
    }
    nonfinite_kernel<<<(n + 255) / 256, 256, 0, stream>>>(pos, vel, n, out);
    return cudaGetLastError();
}

cudaError_t launch_features(const float4* spos2, const float4* svel, const uint32_t* sorted_ids, const uint2* bucket,
                            const TankConst* tanks, const uint16_t* stank, uint32_t n, const uint32_t* order,
                            const uint32_t* masks, float4* force, float* features, bool id_order,
                            cudaStream_t stream, const float* norm_mean, const float* norm_inv_std,
                            uint8_t* x_tiles) {
    if (n == 0) {
        return cudaSuccess;
    }
    // Seven blocks per SM (72 registers) rather than six at the 80 it takes unbounded.
    features_kernel<128, 48, 7><<<(n + 127) / 128, 128, 0, stream>>>(spos2, svel, sorted_ids, bucket, tanks, stank, n,
                                                                     order, masks, force, features, id_order ? 1 : 0,
                                                                     norm_mean, norm_inv_std, x_tiles);
    return cudaGetLastError();
}

namespace {

// A launch that may begin while the kernel before it in the stream finishes
// (programmatic stream serialisation); the kernel waits for that grid's end
// (griddepcontrol.wait) before it reads what the grid wrote.
template <typename Kernel, typename... Args>
cudaError_t launch_after(bool programmatic, dim3 grid, dim3 block, size_t smem, cudaStream_t stream, Kernel kernel,
                         Args... args) {
    cudaLaunchAttribute attr{};
    attr.id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr.val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cfg.attrs = programmatic ? &attr : nullptr;
    cfg.numAttrs = programmatic ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, kernel, args...);
}

}  // namespace

cudaError_t zero_correction_sums(uint32_t tank_count, unsigned long long* sums, cudaStream_t stream) {
    return cudaMemsetAsync(sums, 0, sizeof(unsigned long long) * kCorrectionSumWords * tank_count, stream);
}

cudaError_t launch_correction_sums(const float4* correction, const TankConst* tanks, const uint16_t* stank, uint32_t n,
                                   uint32_t tank_count, unsigned long long* sums, cudaStream_t stream,
                                   bool programmatic) {
    if (!programmatic) {
        const cudaError_t e = zero_correction_sums(tank_count, sums, stream);
        if (e != cudaSuccess) {
            return e;
        }
    }
    if (n == 0) {
        return cudaSuccess;
    }
    int device = 0;
    int sms = 152;
    if (cudaGetDevice(&device) == cudaSuccess) {
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    }
    const uint32_t blocks = std::min<uint32_t>((n + 255) / 256, 4u * static_cast<uint32_t>(sms));
    return launch_after(programmatic, dim3(blocks), dim3(256), 0, stream, correction_sums_kernel, correction, tanks,
                        stank, n, sums);
}

cudaError_t launch_finish_learned(const float4* spos2, const float4* svel, const uint32_t* sorted_ids,
                                  const TankConst* tanks, const uint16_t* stank, uint32_t n, const float4* force,
                                  const float4* correction, const unsigned long long* sums, uint32_t free_axes,
                                  float4* pos, float4* vel, cudaStream_t stream, bool programmatic) {
    if (n == 0) {
        return cudaSuccess;
    }
    return launch_after(programmatic, dim3((n + 255) / 256), dim3(256), 0, stream, finish_learned_kernel, spos2, svel,
                        sorted_ids, tanks, stank, n, force, correction, sums, free_axes, pos, vel);
}

cudaError_t launch_division_selftest(uint64_t seed, uint64_t count, int mode, unsigned long long* mismatches,
                                     cudaStream_t stream) {
    division_selftest_kernel<<<152 * 8, 256, 0, stream>>>(seed, count, mode, mismatches);
    return cudaGetLastError();
}

cudaError_t launch_bucket_stats(const uint2* bucket, uint32_t buckets, uint32_t* out2, cudaStream_t stream) {
    if (buckets == 0) {
        return cudaSuccess;
    }
    bucket_stats_kernel<<<(buckets + 255) / 256, 256, 0, stream>>>(bucket, buckets, out2);
    return cudaGetLastError();
}

}  // namespace sph
