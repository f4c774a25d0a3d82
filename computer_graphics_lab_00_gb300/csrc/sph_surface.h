// sph_surface.h — device fluid surface: field sampling and marching cubes
// (physics::buildFluidField / physics::marchFluidField).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/sph_c.h"

namespace sph {
namespace surface {

// Sample grid of buildFluidField: (resolution + 1)^3 samples at
// origin + (x, y, z) * cell, kernel radius = the smoothing radius.
struct FieldGeom {
    float origin[3];
    float cell[3];
    float radius;
    float radius_sq;  // radius * radius
    uint32_t mask;    // bucket count - 1
    uint32_t resolution;
};

// The interior samples along one axis that fall in one grid cell (the
// mapping sample -> cell is monotone per axis): x in [begin, end).
struct AxisRun {
    uint32_t begin;
    uint32_t end;
    int32_t cell;
    uint32_t pad;
};

// Device scratch of one field: the runs of the three axes.
struct FieldRuns {
    uint32_t count[4];
    AxisRun run[3][SPH_SURFACE_MAX_RESOLUTION];
};

// Arguments of marchFluidField.
struct MarchGeom {
    float origin[3];
    float cell[3];
    float iso;
    uint32_t resolution;
};

// Device scratch of one march: a case code per cell, per-tile totals and
// offsets (march_tiles(resolution) + 1 entries), and the overflow slot.
struct MarchScratch {
    uint8_t* codes;
    uint32_t* tile_sums;
    uint32_t* offsets;
    uint32_t* limit;
};

// The generated case table (256 x SPH_MC_TABLE_WIDTH, -1 ends a case).
const int8_t* case_table();
// Uploads the table to the current device once.
cudaError_t ensure_tables();
uint32_t march_tiles(uint32_t resolution);

// Zeroes the field, splits each axis into per-cell runs, then samples every
// grid cell's box of interior samples with one warp.
cudaError_t launch_field(const float4* spos, const uint2* bucket, const FieldGeom& g, FieldRuns* runs, float* field,
                         cudaStream_t stream);
// After it: vertex count = min(offsets[tiles], *limit).
cudaError_t launch_march(const float* field, const MarchGeom& g, uint32_t capacity, MarchScratch s,
                         sph_surface_vertex* out, cudaStream_t stream);

}  // namespace surface
}  // namespace sph
