// sph_instances.cu — per-particle draw instances for a renderer, written on
// the device (shaders/fluid_instances.comp; CPU twin src/gfx/fluid.cpp:402-466).
#include <cuda_runtime.h>

#include "sph_instances.h"

namespace sph {

namespace {

// One instance (and TLAS record) per particle. The model matrix is
// scale(translate(I, p), r): radius on the diagonal, position in column 3.
//
// Each warp writes the contiguous output of its 32 particles: 14 16-byte
// pieces per instance and 4 per TLAS record, piece k of the warp's region
// going to lane k mod 32, so every store instruction covers 512 consecutive
// bytes. A lane that needs a position reads it from the particle arrays
// (the warp's 32 positions share four cache lines). keepRendered is fused
// in: once its lanes have read the previous positions, the warp copies its
// current positions over them.
constexpr uint32_t kInstancePieces = sizeof(sph_instance) / 16;
constexpr uint32_t kTlasPieces = sizeof(sph_tlas_instance) / 16;
static_assert(sizeof(sph_instance) == 224 && sizeof(sph_tlas_instance) == 64, "record layouts");

__device__ __forceinline__ float pick(uint32_t axis, uint32_t want, float v) { return axis == want ? v : 0.0f; }

__device__ __forceinline__ uint4 as_uint4(float x, float y, float z, float w) {
    return make_uint4(__float_as_uint(x), __float_as_uint(y), __float_as_uint(z), __float_as_uint(w));
}

// Piece e (0..13) of an instance: model rows 0-3, previous model rows 4-7,
// normal matrix (identity: uniform scale) rows 8-11, the index words 12-13.
__device__ __forceinline__ uint4 instance_piece(uint32_t e, const float4* __restrict__ pos,
                                                const float4* prev, uint32_t i, float radius,
                                                uint32_t sphere_mesh, uint32_t flags) {
    if (e == 12) {
        return make_uint4(sphere_mesh, 0u, 0u, SPH_NO_JOINTS);
    }
    if (e == 13) {
        return make_uint4(SPH_NO_JOINTS, SPH_NO_JOINTS, 0u, 0u);
    }
    if (e == 3 || e == 7) {
        const float4 c = (e == 7 && (flags & SPH_INSTANCES_RESET_HISTORY) == 0) ? prev[i] : pos[i];
        return as_uint4(c.x, c.y, c.z, 1.0f);
    }
    const uint32_t row = e & 3u;
    const float s = e < 8 ? radius : 1.0f;
    return as_uint4(pick(row, 0, s), pick(row, 1, s), pick(row, 2, s), pick(row, 3, s));
}

// Piece u (0..3) of a TLAS record: transform rows 0-2, then the index,
// flags and acceleration-structure words.
__device__ __forceinline__ uint4 tlas_piece(uint32_t u, const float4* __restrict__ pos, uint32_t i, float radius,
                                            uint32_t slot, unsigned long long blas, uint32_t fluid_index,
                                            uint32_t flags) {
    const uint32_t lo = static_cast<uint32_t>(blas), hi = static_cast<uint32_t>(blas >> 32);
    if ((flags & SPH_INSTANCES_SURFACE_TLAS) != 0) {
        // Surface mode: record 0 is the surface (world-space vertices, identity
        // transform, shadow-ray mask, culling off); the others are inactive.
        const bool first = i == 0;
        if (u == 3) {
            return first ? make_uint4((SPH_FLUID_SURFACE_CUSTOM_INDEX | fluid_index) | (SPH_FLUID_SURFACE_RAY_MASK << 24u),
                                      1u << 24u, lo, hi)
                         : make_uint4(0u, 0u, 0u, 0u);
        }
        const float one = first ? 1.0f : 0.0f;
        return as_uint4(pick(u, 0, one), pick(u, 1, one), pick(u, 2, one), 0.0f);
    }
    if (u == 3) {
        return make_uint4((slot & 0xFFFFFFu) | (0xFFu << 24u), 0u, lo, hi);
    }
    const float4 p = pos[i];
    const float t = u == 0 ? p.x : (u == 1 ? p.y : p.z);
    return as_uint4(pick(u, 0, radius), pick(u, 1, radius), pick(u, 2, radius), t);
}

__global__ void __launch_bounds__(256) instances_kernel(const float4* __restrict__ pos,
                                                        float4* __restrict__ prev, uint32_t n, float radius,
                                                        sph_instance* __restrict__ instances, uint32_t instance_base,
                                                        uint32_t sphere_mesh, sph_tlas_instance* __restrict__ tlas,
                                                        uint32_t tlas_base, unsigned long long blas,
                                                        uint32_t fluid_index, uint32_t flags) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t first = (blockIdx.x * blockDim.x + threadIdx.x) - lane;
    if (first >= n) {
        return;
    }
    const uint32_t count = min(32u, n - first);
    uint4* out = reinterpret_cast<uint4*>(instances + instance_base + first);
    for (uint32_t k = lane; k < count * kInstancePieces; k += 32) {
        const uint32_t j = k / kInstancePieces;
        out[k] = instance_piece(k - j * kInstancePieces, pos, prev, first + j, radius, sphere_mesh, flags);
    }
    if ((flags & SPH_INSTANCES_WRITE_TLAS) != 0) {
        uint4* rec = reinterpret_cast<uint4*>(tlas + tlas_base + first);
        for (uint32_t k = lane; k < count * kTlasPieces; k += 32) {
            const uint32_t j = k / kTlasPieces;
            rec[k] = tlas_piece(k % kTlasPieces, pos, first + j, radius, instance_base + first + j, blas, fluid_index,
                                flags);
        }
    }
    __syncwarp();
    if (lane < count) {
        prev[first + lane] = pos[first + lane];
    }
}

}  // namespace

cudaError_t launch_instances(const float4* pos, float4* prev, uint32_t n, float radius, sph_instance* instances,
                             uint32_t instance_base, uint32_t sphere_mesh, sph_tlas_instance* tlas, uint32_t tlas_base,
                             unsigned long long blas, uint32_t fluid_index, uint32_t flags, cudaStream_t stream) {
    if (n == 0) {
        return cudaSuccess;
    }
    instances_kernel<<<(n + 255) / 256, 256, 0, stream>>>(pos, prev, n, radius, instances, instance_base, sphere_mesh,
                                                          tlas, tlas_base, blas, fluid_index, flags);
    return cudaGetLastError();
}

}  // namespace sph
