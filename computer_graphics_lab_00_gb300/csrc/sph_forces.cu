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

namespace sph {

namespace {

// std::max(a, b) returns b only when a < b.
__device__ __forceinline__ float max_like_std(float a, float b) { return a < b ? b : a; }

template <bool kCount>
__global__ void __launch_bounds__(128) density_kernel(const float4* __restrict__ spos, float4* __restrict__ svel,
                                                      float4* __restrict__ spos2, const uint2* __restrict__ bucket,
                                                      const TankConst* __restrict__ tanks,
                                                      const uint16_t* __restrict__ stank, uint32_t n,
                                                      StepCounters* __restrict__ counters) {
    uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
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
                                                        const uint16_t* __restrict__ stank, uint32_t n,
                                                        float4* __restrict__ pos_out, float4* __restrict__ vel_out) {
    uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
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

    // fluid_sph.cpp:260-285. The force-field sum starts at vec3{0} and is
    // added even when there are no fields, which maps -0 to +0.
    const float dt = __ldg(&t->dt);
    float ax = __fadd_rn(__fadd_rn(__fdiv_rn(fx, density), __ldg(&t->gravity[0])), 0.0f);
    float ay = __fadd_rn(__fadd_rn(__fdiv_rn(fy, density), __ldg(&t->gravity[1])), 0.0f);
    float az = __fadd_rn(__fadd_rn(__fdiv_rn(fz, density), __ldg(&t->gravity[2])), 0.0f);
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
    uint32_t i = sorted_ids[p];
    pos_out[i] = make_float4(pp[0], pp[1], pp[2], density);
    vel_out[i] = make_float4(vv[0], vv[1], vv[2], pressure);
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

// Per-tank FP64 sums. Lanes of a warp that belong to one tank reduce with
// shuffles; a warp that straddles tanks falls back to per-lane atomics.
__global__ void stats_kernel(const float4* __restrict__ pos, const float4* __restrict__ vel,
                             const uint16_t* __restrict__ tank_of, const TankConst* __restrict__ tanks, uint32_t n,
                             double* __restrict__ acc) {
    uint32_t stride = gridDim.x * blockDim.x;
    uint32_t lane = threadIdx.x & 31;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += stride) {
        uint32_t i = base + threadIdx.x;
        bool valid = i < n;
        uint32_t tank = valid && tank_of != nullptr ? tank_of[i] : 0;
        double v[kStatsPerTank] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
        if (valid) {
            float4 p = pos[i];
            float4 u = vel[i];
            const TankConst* t = tanks + tank;
            double rho0 = t->rest_density;
            double rho = p.w;
            bool finite = isfinite(p.x) && isfinite(p.y) && isfinite(p.z) && isfinite(u.x) && isfinite(u.y) &&
                          isfinite(u.z);
            v[0] = rho;
            v[1] = fmax(0.0, rho - rho0) / rho0;
            v[2] = rho;
            v[3] = p.x;
            v[4] = p.y;
            v[5] = p.z;
            v[6] = 0.5 * static_cast<double>(t->mass) *
                   (static_cast<double>(u.x) * u.x + static_cast<double>(u.y) * u.y + static_cast<double>(u.z) * u.z);
            v[7] = finite ? 0.0 : 1.0;
            v[8] = 1.0;
        }
        uint32_t key = valid ? tank : 0xFFFFFFFFu;
        uint32_t peers = __match_any_sync(0xFFFFFFFFu, key);
        double* dst = acc + static_cast<size_t>(tank) * kStatsPerTank;
        if (peers == 0xFFFFFFFFu && valid) {
            double s[kStatsPerTank];
#pragma unroll
            for (int k = 0; k < static_cast<int>(kStatsPerTank); ++k) {
                s[k] = k == 2 ? warp_max(v[k]) : warp_sum(v[k]);
            }
            if (lane == 0) {
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
        } else if (valid) {
            for (int k = 0; k < static_cast<int>(kStatsPerTank); ++k) {
                if (k == 2) {
                    atomicMax(reinterpret_cast<unsigned long long*>(dst + 2),
                              static_cast<unsigned long long>(__double_as_longlong(fmax(v[2], 0.0))));
                } else if (k != 9) {
                    atomicAdd(dst + k, v[k]);
                }
            }
        }
    }
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

}  // namespace

cudaError_t launch_density(const float4* spos, float4* svel, float4* spos2, const uint2* bucket, const TankConst* tanks,
                           const uint16_t* stank, uint32_t n, StepCounters* counters, cudaStream_t stream) {
    if (n == 0) {
        return cudaSuccess;
    }
    uint32_t blocks = (n + 127) / 128;
    if (counters != nullptr) {
        density_kernel<true><<<blocks, 128, 0, stream>>>(spos, svel, spos2, bucket, tanks, stank, n, counters);
    } else {
        density_kernel<false><<<blocks, 128, 0, stream>>>(spos, svel, spos2, bucket, tanks, stank, n, nullptr);
    }
    return cudaGetLastError();
}

cudaError_t launch_integrate(const float4* spos2, const float4* svel, const uint32_t* sorted_ids, const uint2* bucket,
                             const TankConst* tanks, const uint16_t* stank, uint32_t n, float4* pos, float4* vel,
                             cudaStream_t stream) {
    if (n == 0) {
        return cudaSuccess;
    }
    integrate_kernel<<<(n + 127) / 128, 128, 0, stream>>>(spos2, svel, sorted_ids, bucket, tanks, stank, n, pos, vel);
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
    uint32_t blocks = (n + 255) / 256;
    if (blocks > 4 * 152) {
        blocks = 4 * 152;
    }
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

cudaError_t launch_bucket_stats(const uint2* bucket, uint32_t buckets, uint32_t* out2, cudaStream_t stream) {
    if (buckets == 0) {
        return cudaSuccess;
    }
    bucket_stats_kernel<<<(buckets + 255) / 256, 256, 0, stream>>>(bucket, buckets, out2);
    return cudaGetLastError();
}

}  // namespace sph
