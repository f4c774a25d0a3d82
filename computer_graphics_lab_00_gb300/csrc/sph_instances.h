// sph_instances.h — device instance writer (see sph_instances.cu).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/sph_c.h"

namespace sph {

// Writes the instances (and TLAS records) of particles [0, n) and then
// copies pos[0, n) over prev[0, n) (keepRendered for those particles).
cudaError_t launch_instances(const float4* pos, float4* prev, uint32_t n, float radius, sph_instance* instances,
                             uint32_t instance_base, uint32_t sphere_mesh, sph_tlas_instance* tlas, uint32_t tlas_base,
                             unsigned long long blas, uint32_t fluid_index, uint32_t flags, cudaStream_t stream);

}  // namespace sph
