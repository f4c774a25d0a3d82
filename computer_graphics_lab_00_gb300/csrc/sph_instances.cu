// sph_instances.cu — per-particle draw instances for a renderer, written on
// the device (shaders/fluid_instances.comp; CPU twin src/gfx/fluid.cpp:402-466).
#include <cuda_runtime.h>

#include "sph_instances.h"

namespace sph {

namespace {

// One instance (and TLAS record) per particle. The model matrix is
// scale(translate(I, p), r): radius on the diagonal, position in column 3.
__global__ void __launch_bounds__(256) instances_kernel(const float4* __restrict__ pos,
                                                        const float4* __restrict__ prev, uint32_t n, float radius,
                                                        sph_instance* __restrict__ instances, uint32_t instance_base,
                                                        uint32_t sphere_mesh, sph_tlas_instance* __restrict__ tlas,
                                                        uint32_t tlas_base, unsigned long long blas,
                                                        uint32_t fluid_index, uint32_t flags) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) {
        return;
    }
    const float4 p = pos[i];
    const float4 q = (flags & SPH_INSTANCES_RESET_HISTORY) != 0 ? p : prev[i];
    const uint32_t slot = instance_base + i;
    float4* out = reinterpret_cast<float4*>(instances + slot);
    // model, previous model, normal matrix (identity: uniform scale).
    out[0] = make_float4(radius, 0.0f, 0.0f, 0.0f);
    out[1] = make_float4(0.0f, radius, 0.0f, 0.0f);
    out[2] = make_float4(0.0f, 0.0f, radius, 0.0f);
    out[3] = make_float4(p.x, p.y, p.z, 1.0f);
    out[4] = make_float4(radius, 0.0f, 0.0f, 0.0f);
    out[5] = make_float4(0.0f, radius, 0.0f, 0.0f);
    out[6] = make_float4(0.0f, 0.0f, radius, 0.0f);
    out[7] = make_float4(q.x, q.y, q.z, 1.0f);
    out[8] = make_float4(1.0f, 0.0f, 0.0f, 0.0f);
    out[9] = make_float4(0.0f, 1.0f, 0.0f, 0.0f);
    out[10] = make_float4(0.0f, 0.0f, 1.0f, 0.0f);
    out[11] = make_float4(0.0f, 0.0f, 0.0f, 1.0f);
    uint4* tail = reinterpret_cast<uint4*>(out + 12);
    tail[0] = make_uint4(sphere_mesh, 0u, 0u, SPH_NO_JOINTS);
    tail[1] = make_uint4(SPH_NO_JOINTS, SPH_NO_JOINTS, 0u, 0u);
    if ((flags & SPH_INSTANCES_WRITE_TLAS) != 0) {
        sph_tlas_instance t;
        if ((flags & SPH_INSTANCES_SURFACE_TLAS) != 0) {
            // Surface mode: record 0 is the surface (world-space vertices, identity
            // transform, shadow-ray mask, culling off); the others are inactive.
            const bool first = i == 0;
            const float one = first ? 1.0f : 0.0f;
            const float rows[12] = {one, 0.0f, 0.0f, 0.0f, 0.0f, one, 0.0f, 0.0f, 0.0f, 0.0f, one, 0.0f};
            for (int k = 0; k < 12; ++k) {
                t.transform[k] = rows[k];
            }
            t.custom_index_mask =
                first ? ((SPH_FLUID_SURFACE_CUSTOM_INDEX | fluid_index) | (SPH_FLUID_SURFACE_RAY_MASK << 24u)) : 0u;
            t.sbt_offset_flags = first ? (1u << 24u) : 0u;
            t.blas = first ? blas : 0ull;
        } else {
            const float rows[12] = {radius, 0.0f, 0.0f, p.x, 0.0f, radius, 0.0f, p.y, 0.0f, 0.0f, radius, p.z};
            for (int k = 0; k < 12; ++k) {
                t.transform[k] = rows[k];
            }
            t.custom_index_mask = (slot & 0xFFFFFFu) | (0xFFu << 24u);
            t.sbt_offset_flags = 0u;
            t.blas = blas;
        }
        tlas[tlas_base + i] = t;
    }
}

}  // namespace

cudaError_t launch_instances(const float4* pos, const float4* prev, uint32_t n, float radius, sph_instance* instances,
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
