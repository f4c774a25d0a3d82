// sph_surface.cu — the fluid surface on the device: the scalar field of
// physics::buildFluidField and the marching cubes of physics::marchFluidField
// (src/physics/marching_cubes.cpp:300-483, src/asset/vertex_pack.h:20-51).
//
// Every float expression follows the reference operation by operation; this
// translation unit is compiled with --fmad=false. Vertices come out in the
// reference's serial order (cell index, then the case's table order): a count
// pass writes each cell's case code and its block's vertex total, a scan of
// the block totals gives each block its first slot, and the emit pass scans
// its block again to place every cell. A cell whose vertices would pass the
// capacity is dropped together with every later cell, as in the reference.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>

#include "../../include/sph_c.h"
#include "sph_device.cuh"
#include "sph_surface.h"

namespace sph {
namespace surface {

// ---- the case table -----------------------------------------------------------------
//
// Built from the rule the reference documents for its MC_TABLE
// (marching_cubes.cpp:18-24): the contour on a cell face depends only on
// that face's four corner signs, an ambiguous face (two diagonal corners
// inside) wraps each inside corner on its own, and triangles face from the
// inside corners towards the outside ones. Each contour loop is traced from
// its lowest-numbered edge, first across the lower-numbered of that edge's
// two faces, turned outward, and fanned from its first edge; loops are
// emitted in order of their lowest edge. Corner and edge numbering are the
// reference's (MC_CORNERS, MC_EDGES).

namespace {

constexpr int kCorner[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0}, {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
constexpr int kEdge[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {4, 5}, {5, 6}, {6, 7}, {7, 4}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};
// Cell faces as corner cycles: z = 0, z = 1, y = 0, y = 1, x = 0, x = 1.
constexpr int kFace[6][4] = {{0, 1, 2, 3}, {4, 5, 6, 7}, {0, 1, 5, 4}, {3, 2, 6, 7}, {0, 3, 7, 4}, {1, 2, 6, 5}};

struct Tables {
    int8_t entry[256][SPH_MC_TABLE_WIDTH];
    uint8_t count[256];
};

Tables generate() {
    Tables t{};
    // face_edge[f][k]: the edge between corners k and k+1 of face f.
    int face_edge[6][4];
    for (int f = 0; f < 6; ++f) {
        for (int k = 0; k < 4; ++k) {
            int a = kFace[f][k];
            int b = kFace[f][(k + 1) & 3];
            for (int e = 0; e < 12; ++e) {
                if ((kEdge[e][0] == a && kEdge[e][1] == b) || (kEdge[e][0] == b && kEdge[e][1] == a)) {
                    face_edge[f][k] = e;
                }
            }
        }
    }
    // The two faces of every edge, lower face first.
    int edge_face[12][2];
    int seen_faces[12] = {};
    for (int f = 0; f < 6; ++f) {
        for (int k = 0; k < 4; ++k) {
            int e = face_edge[f][k];
            edge_face[e][seen_faces[e]++] = f;
        }
    }
    for (int code = 0; code < 256; ++code) {
        auto in = [code](int corner) { return ((code >> corner) & 1) != 0; };
        uint32_t active = 0;
        for (int e = 0; e < 12; ++e) {
            if (in(kEdge[e][0]) != in(kEdge[e][1])) {
                active |= 1u << e;
            }
        }
        // Across face f from active edge e: walk the face's edge cycle from e
        // towards e's inside corner to the next active edge.
        auto across = [&](int f, int e) {
            int k = 0;
            while (face_edge[f][k] != e) {
                ++k;
            }
            const int step = in(kFace[f][(k + 1) & 3]) ? 1 : 3;
            do {
                k = (k + step) & 3;
            } while ((active >> face_edge[f][k] & 1u) == 0);
            return face_edge[f][k];
        };
        uint32_t done = 0;
        int n = 0;
        for (int first = 0; first < 12; ++first) {
            if ((active >> first & 1u) == 0 || (done >> first & 1u) != 0) {
                continue;
            }
            int loop[12];
            int len = 0;
            int face = edge_face[first][0];
            int e = first;
            do {
                loop[len++] = e;
                done |= 1u << e;
                int next = across(face, e);
                face = edge_face[next][0] == face ? edge_face[next][1] : edge_face[next][0];
                e = next;
            } while (e != first);
            // Orientation: the loop's area vector (over edge midpoints, in
            // half units) against the summed inside-to-outside edge directions.
            long area[3] = {0, 0, 0};
            long outward[3] = {0, 0, 0};
            for (int i = 0; i < len; ++i) {
                int a = loop[i];
                int b = loop[(i + 1) % len];
                long ma[3], mb[3];
                for (int d = 0; d < 3; ++d) {
                    ma[d] = kCorner[kEdge[a][0]][d] + kCorner[kEdge[a][1]][d];
                    mb[d] = kCorner[kEdge[b][0]][d] + kCorner[kEdge[b][1]][d];
                }
                area[0] += ma[1] * mb[2] - ma[2] * mb[1];
                area[1] += ma[2] * mb[0] - ma[0] * mb[2];
                area[2] += ma[0] * mb[1] - ma[1] * mb[0];
                int inner = in(kEdge[a][0]) ? kEdge[a][0] : kEdge[a][1];
                int outer = inner == kEdge[a][0] ? kEdge[a][1] : kEdge[a][0];
                for (int d = 0; d < 3; ++d) {
                    outward[d] += kCorner[outer][d] - kCorner[inner][d];
                }
            }
            if (area[0] * outward[0] + area[1] * outward[1] + area[2] * outward[2] < 0) {
                std::reverse(loop, loop + len);
            }
            for (int i = 1; i + 1 < len; ++i) {
                t.entry[code][n++] = static_cast<int8_t>(loop[0]);
                t.entry[code][n++] = static_cast<int8_t>(loop[i]);
                t.entry[code][n++] = static_cast<int8_t>(loop[i + 1]);
            }
        }
        t.count[code] = static_cast<uint8_t>(n);
        for (int i = n; i < static_cast<int>(SPH_MC_TABLE_WIDTH); ++i) {
            t.entry[code][i] = -1;
        }
    }
    return t;
}

const Tables& tables() {
    static const Tables t = generate();
    return t;
}

// The case table and vertex counts sit in global memory and the march kernels
// stage them in shared memory: the lanes of a warp look up different cases,
// which constant memory would serve one address at a time.
__device__ int8_t g_entry[256][SPH_MC_TABLE_WIDTH];
__device__ uint8_t g_count[256];
__constant__ int8_t c_corner[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                                      {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};

// Corner c of a cell (the corner table above, as bits) and the corners of
// edge e: the four bottom edges (0-1, 1-2, 2-3, 3-0), the four top edges
// (4-5, 5-6, 6-7, 7-4), then the four verticals (0-4, 1-5, 2-6, 3-7).
__device__ __forceinline__ int corner_offset(int c, int d) {
    return d == 0 ? ((c ^ (c >> 1)) & 1) : (d == 1 ? ((c >> 1) & 1) : (c >> 2));
}
__device__ __forceinline__ void edge_corners(int e, int& a, int& b) {
    if (e < 8) {
        a = e;
        b = (e & 4) | ((e + 1) & 3);
    } else {
        a = e - 8;
        b = e - 4;
    }
}

constexpr uint32_t kBlock = 256;
constexpr uint32_t kPerThread = 8;
constexpr uint32_t kTile = kBlock * kPerThread;  // cells per count/emit block

// ---- field ------------------------------------------------------------------------

// sampleField (marching_cubes.cpp:312-347) at every interior sample; border
// samples are 0 (buildFluidField, :380-391).
//
// Every sample of one grid cell (cell size = the kernel radius) visits the
// same 27 buckets, so the samples are grouped by cell: along each axis the
// sample -> cell map is monotone, so a cell's samples form a box of per-axis
// runs, and one warp takes a box. Its lanes walk the buckets in step (one
// broadcast load per candidate, no divergent trip counts), kPer samples per
// lane. Each sample still sums its candidates in the reference's order.

// Per-axis runs of interior samples [1, resolution) with the same cell.
__global__ void __launch_bounds__(1024) field_runs_kernel(FieldGeom g, FieldRuns* __restrict__ runs) {
    __shared__ int32_t cells[SPH_SURFACE_MAX_RESOLUTION + 1];
    const uint32_t a = blockIdx.x;
    const uint32_t r = g.resolution;
    const float origin = a == 0 ? g.origin[0] : (a == 1 ? g.origin[1] : g.origin[2]);
    const float cell = a == 0 ? g.cell[0] : (a == 1 ? g.cell[1] : g.cell[2]);
    for (uint32_t x = 1 + threadIdx.x; x < r; x += blockDim.x) {
        // origin + float(x) * cell, as the sample position.
        cells[x] = cell_coord(__fadd_rn(origin, __fmul_rn(static_cast<float>(x), cell)), g.radius);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t n = 0;
        for (uint32_t x = 1; x < r; ++x) {
            if (x == 1 || cells[x] != cells[x - 1]) {
                if (n > 0) {
                    runs->run[a][n - 1].end = x;
                }
                runs->run[a][n] = AxisRun{x, x, cells[x], 0u};
                ++n;
            }
        }
        if (n > 0) {
            runs->run[a][n - 1].end = r;
        }
        runs->count[a] = n;
    }
}

// kGroup lanes (8, 16 or 32) share one box; a warp holds 32 / kGroup boxes.
// Lane j of a group hashes neighbours j, j + kGroup, ... and the group reads
// them back by shuffle.
template <int kGroup, int kPer>
__global__ void __launch_bounds__(kBlock) field_cells_kernel(const float4* __restrict__ spos,
                                                             const uint2* __restrict__ bucket, FieldGeom g,
                                                             const FieldRuns* __restrict__ runs,
                                                             float* __restrict__ field) {
    static_assert(kGroup == 8 || kGroup == 16 || kGroup == 32, "group of 8, 16 or 32 lanes");
    constexpr uint32_t kAll = 0xFFFFFFFFu;
    constexpr int kSlots = (27 + kGroup - 1) / kGroup;  // neighbours per lane
    constexpr uint32_t kGroupsPerWarp = 32u / kGroup;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t glane = lane % kGroup;
    const uint32_t gbase = lane - glane;
    const uint32_t nx = runs->count[0];
    const uint32_t ny = runs->count[1];
    const uint32_t nz = runs->count[2];
    const uint32_t boxes = nx * ny * nz;
    const uint32_t samples = g.resolution + 1;
    const uint32_t warps = gridDim.x * (kBlock / 32u);
    const uint32_t warp_id = blockIdx.x * (kBlock / 32u) + (threadIdx.x >> 5);
    const uint32_t rounds = (boxes + warps * kGroupsPerWarp - 1) / (warps * kGroupsPerWarp);
    for (uint32_t round = 0; round < rounds; ++round) {
        // Every lane stays in the loop (the shuffles need the whole warp); a
        // group past the last box works on box 0 and writes nothing.
        const uint32_t w = (round * warps + warp_id) * kGroupsPerWarp + lane / kGroup;
        const bool live = w < boxes;
        const uint32_t box = live ? w : 0u;
        const AxisRun rx = runs->run[0][box % nx];
        const AxisRun ry = runs->run[1][(box / nx) % ny];
        const AxisRun rz = runs->run[2][box / (nx * ny)];
        // The 27 buckets in (z, y, x) order; a bucket reached twice (two
        // cells that hash alike) is summed once, at its first offset.
        uint32_t h[kSlots];
        uint2 range[kSlots];
#pragma unroll
        for (int t = 0; t < kSlots; ++t) {
            const uint32_t k = glane + static_cast<uint32_t>(t) * kGroup;
            h[t] = 0xFFFFFFFFu;
            if (k < 27u) {
                const int dx = static_cast<int>(k % 3u) - 1;
                const int dy = static_cast<int>((k / 3u) % 3u) - 1;
                const int dz = static_cast<int>(k / 9u) - 1;
                h[t] = spatial_hash(static_cast<uint32_t>(rx.cell + dx), static_cast<uint32_t>(ry.cell + dy),
                                    static_cast<uint32_t>(rz.cell + dz), g.mask);
            }
            range[t] = k < 27u ? __ldg(&bucket[h[t]]) : make_uint2(0u, 0u);
        }
        uint32_t skip = 0;  // bit k: neighbour k repeats an earlier bucket
#pragma unroll
        for (int t = 0; t < kSlots; ++t) {
            const uint32_t k = glane + static_cast<uint32_t>(t) * kGroup;
            bool repeat = false;
#pragma unroll
            for (uint32_t j = 0; j < 27u; ++j) {
                const uint32_t bj = __shfl_sync(kAll, h[j / kGroup], static_cast<int>(gbase + j % kGroup));
                repeat = repeat || (j < k && bj == h[t]);
            }
            const uint32_t votes = __ballot_sync(kAll, k < 27u && repeat);
            skip |= ((votes >> gbase) & (kGroup == 32 ? kAll : ((1u << kGroup) - 1u))) << (t * kGroup);
        }
        const uint32_t bw = rx.end - rx.begin;
        const uint32_t bh = ry.end - ry.begin;
        const uint32_t n_box = bw * bh * (rz.end - rz.begin);
        // Passes over the box; a group with fewer samples idles through the
        // extra passes of a bigger box in its warp.
        const uint32_t my_passes = (n_box + kGroup * kPer - 1) / (kGroup * kPer);
        uint32_t passes = my_passes;
#pragma unroll
        for (uint32_t o = kGroup; o < 32u; o <<= 1) {
            passes = max(passes, __shfl_xor_sync(kAll, passes, static_cast<int>(o)));
        }
        for (uint32_t pass = 0; pass < passes; ++pass) {
            const uint32_t first = pass * kGroup * kPer;
            float px[kPer];
            float py[kPer];
            float pz[kPer];
            float sum[kPer];
#pragma unroll
            for (int q = 0; q < kPer; ++q) {
                const uint32_t i = min(first + static_cast<uint32_t>(q) * kGroup + glane, n_box - 1u);
                const uint32_t x = rx.begin + i % bw;
                const uint32_t y = ry.begin + (i / bw) % bh;
                const uint32_t z = rz.begin + i / (bw * bh);
                // origin + vec3{x, y, z} * cell.
                px[q] = __fadd_rn(g.origin[0], __fmul_rn(static_cast<float>(x), g.cell[0]));
                py[q] = __fadd_rn(g.origin[1], __fmul_rn(static_cast<float>(y), g.cell[1]));
                pz[q] = __fadd_rn(g.origin[2], __fmul_rn(static_cast<float>(z), g.cell[2]));
                sum[q] = 0.0f;
            }
            for (uint32_t k = 0; k < 27u; ++k) {
                const int src = static_cast<int>(gbase + k % kGroup);
                uint2 held = range[0];  // this lane's slot k / kGroup, without a dynamic index
#pragma unroll
                for (int t = 1; t < kSlots; ++t) {
                    if (k >= static_cast<uint32_t>(t) * kGroup) {
                        held = range[t];
                    }
                }
                const uint32_t start = __shfl_sync(kAll, held.x, src);
                const uint32_t end = __shfl_sync(kAll, held.y, src);
                if ((skip >> k & 1u) != 0 || pass >= my_passes) {
                    continue;
                }
                const uint32_t count = min(end - start, kCellCapacity);
                for (uint32_t s = 0; s < count; ++s) {
                    const float4 p = __ldg(&spos[start + s]);
#pragma unroll
                    for (int q = 0; q < kPer; ++q) {
                        const float ex = __fsub_rn(p.x, px[q]);
                        const float ey = __fsub_rn(p.y, py[q]);
                        const float ez = __fsub_rn(p.z, pz[q]);
                        const float d2 = dot3(ex, ey, ez);
                        if (!(d2 >= g.radius_sq)) {
                            const float d = __fsub_rn(1.0f, __fdiv_rn(d2, g.radius_sq));
                            sum[q] = __fadd_rn(sum[q], __fmul_rn(__fmul_rn(d, d), d));
                        }
                    }
                }
            }
#pragma unroll
            for (int q = 0; q < kPer; ++q) {
                const uint32_t i = first + static_cast<uint32_t>(q) * kGroup + glane;
                if (live && i < n_box) {
                    const uint32_t x = rx.begin + i % bw;
                    const uint32_t y = ry.begin + (i / bw) % bh;
                    const uint32_t z = rz.begin + i / (bw * bh);
                    field[(static_cast<size_t>(z) * samples + y) * samples + x] = sum[q];
                }
            }
        }
    }
}

// ---- marching cubes -----------------------------------------------------------------

// fieldAt (marching_cubes.cpp:350-359): 0 outside the sample grid.
__device__ __forceinline__ float field_at(const float* __restrict__ field, int samples, int x, int y, int z) {
    if (x < 0 || y < 0 || z < 0 || x >= samples || y >= samples || z >= samples) {
        return 0.0f;
    }
    return __ldg(&field[(static_cast<size_t>(z) * samples + y) * samples + x]);
}

__device__ __forceinline__ uint32_t cell_code(const float* __restrict__ field, const MarchGeom& g, uint32_t cell) {
    const int r = static_cast<int>(g.resolution);
    const int s = r + 1;
    const int bx = static_cast<int>(cell % g.resolution);
    const int by = static_cast<int>((cell / g.resolution) % g.resolution);
    const int bz = static_cast<int>(cell / (g.resolution * g.resolution));
    uint32_t code = 0;
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        float v = field_at(field, s, bx + c_corner[c][0], by + c_corner[c][1], bz + c_corner[c][2]);
        code |= (v >= g.iso ? 1u : 0u) << c;
    }
    return code;
}

// Block-wide exclusive scan of one value per thread; returns the block total in *total.
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* total) {
    __shared__ uint32_t warp_sums[kBlock / 32];
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t warp = threadIdx.x >> 5;
    uint32_t inclusive = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        uint32_t up = __shfl_up_sync(0xFFFFFFFFu, inclusive, d);
        if (lane >= static_cast<uint32_t>(d)) {
            inclusive += up;
        }
    }
    if (lane == 31) {
        warp_sums[warp] = inclusive;
    }
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < kBlock / 32 ? warp_sums[lane] : 0u;
        uint32_t wi = w;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            uint32_t up = __shfl_up_sync(0xFFFFFFFFu, wi, d);
            if (lane >= static_cast<uint32_t>(d)) {
                wi += up;
            }
        }
        if (lane < kBlock / 32) {
            warp_sums[lane] = wi - w;  // exclusive prefix of this warp
        }
        if (lane == kBlock / 32 - 1) {
            *total = wi;
        }
    }
    __syncthreads();
    uint32_t out = warp_sums[warp] + inclusive - v;
    __syncthreads();
    return out;
}

// Case code of every cell and the vertex total of every tile of kTile cells.
__global__ void __launch_bounds__(kBlock) count_kernel(const float* __restrict__ field, MarchGeom g,
                                                       uint8_t* __restrict__ codes, uint32_t* __restrict__ tile_sums) {
    static_assert(kBlock == 256, "one thread stages one case's count");
    __shared__ uint8_t s_count[256];
    s_count[threadIdx.x] = g_count[threadIdx.x];
    __syncthreads();
    const uint32_t cells = g.resolution * g.resolution * g.resolution;
    const uint32_t first = blockIdx.x * kTile + threadIdx.x * kPerThread;
    uint32_t sum = 0;
#pragma unroll
    for (uint32_t k = 0; k < kPerThread; ++k) {
        const uint32_t cell = first + k;
        if (cell < cells) {
            const uint32_t code = cell_code(field, g, cell);
            codes[cell] = static_cast<uint8_t>(code);
            sum += s_count[code];
        }
    }
    __shared__ uint32_t total;
    block_exclusive_scan(sum, &total);
    if (threadIdx.x == 0) {
        tile_sums[blockIdx.x] = total;
    }
}

// Exclusive scan of the tile totals in one block; offsets[tiles] = the grand total.
__global__ void __launch_bounds__(1024) tile_scan_kernel(const uint32_t* __restrict__ tile_sums, uint32_t tiles,
                                                         uint32_t* __restrict__ offsets) {
    __shared__ uint32_t part[1024];
    const uint32_t per = (tiles + blockDim.x - 1) / blockDim.x;
    const uint32_t begin = threadIdx.x * per;
    const uint32_t end = min(begin + per, tiles);
    uint32_t sum = 0;
    for (uint32_t t = begin; t < end; ++t) {
        sum += tile_sums[t];
    }
    part[threadIdx.x] = sum;
    __syncthreads();
    // Hillis-Steele over the 1024 partial sums.
    for (uint32_t d = 1; d < blockDim.x; d <<= 1) {
        uint32_t add = threadIdx.x >= d ? part[threadIdx.x - d] : 0u;
        __syncthreads();
        part[threadIdx.x] += add;
        __syncthreads();
    }
    uint32_t run = part[threadIdx.x] - sum;
    for (uint32_t t = begin; t < end; ++t) {
        offsets[t] = run;
        run += tile_sums[t];
    }
    if (threadIdx.x == blockDim.x - 1) {
        offsets[tiles] = part[threadIdx.x];
    }
}

// vertex_pack.h:20-28: lround(clamp(x, -1, 1) * 32767) in 16 bits.
__device__ __forceinline__ uint32_t quantize_snorm16(float x) {
    const float c = x < -1.0f ? -1.0f : (1.0f < x ? 1.0f : x);
    const int32_t q = static_cast<int32_t>(lroundf(__fmul_rn(c, 32767.0f)));
    return static_cast<uint32_t>(q) & 0xFFFFu;
}

// packUnitVector (vertex_pack.h:38-51): octahedral map into two snorm16.
__device__ __forceinline__ uint32_t pack_unit_vector(float x, float y, float z) {
    const float sum = __fadd_rn(__fadd_rn(fabsf(x), fabsf(y)), fabsf(z));
    if (sum <= 0.0f) {
        return 0u;
    }
    x = __fdiv_rn(x, sum);
    y = __fdiv_rn(y, sum);
    z = __fdiv_rn(z, sum);
    float px = x;
    float py = y;
    if (z < 0.0f) {
        px = __fmul_rn(__fsub_rn(1.0f, fabsf(y)), x >= 0.0f ? 1.0f : -1.0f);
        py = __fmul_rn(__fsub_rn(1.0f, fabsf(x)), y >= 0.0f ? 1.0f : -1.0f);
    }
    return quantize_snorm16(px) | (quantize_snorm16(py) << 16u);
}

// Central difference at sample c divided by the cell size (marching_cubes.cpp:451-460).
__device__ __forceinline__ float3 gradient(const float* __restrict__ field, int s, int cx, int cy, int cz,
                                           const MarchGeom& g) {
    const float gx = __fsub_rn(field_at(field, s, cx + 1, cy, cz), field_at(field, s, cx - 1, cy, cz));
    const float gy = __fsub_rn(field_at(field, s, cx, cy + 1, cz), field_at(field, s, cx, cy - 1, cz));
    const float gz = __fsub_rn(field_at(field, s, cx, cy, cz + 1), field_at(field, s, cx, cy, cz - 1));
    return make_float3(__fdiv_rn(gx, g.cell[0]), __fdiv_rn(gy, g.cell[1]), __fdiv_rn(gz, g.cell[2]));
}

// One vertex of a cell (marching_cubes.cpp:418-478): the interpolated point on
// table entry v's edge and the packed outward normal.
__device__ __forceinline__ sph_surface_vertex cell_vertex(const float* __restrict__ field, const MarchGeom& g,
                                                          uint32_t cell, const int8_t* entry, uint32_t v) {
    const int s = static_cast<int>(g.resolution) + 1;
    const int base[3] = {static_cast<int>(cell % g.resolution), static_cast<int>((cell / g.resolution) % g.resolution),
                         static_cast<int>(cell / (g.resolution * g.resolution))};
    int a, b;
    edge_corners(entry[v], a, b);
    int ca[3], cb[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        ca[d] = base[d] + corner_offset(a, d);
        cb[d] = base[d] + corner_offset(b, d);
    }
    const float va = field_at(field, s, ca[0], ca[1], ca[2]);
    const float vb = field_at(field, s, cb[0], cb[1], cb[2]);
    const float diff = __fsub_rn(vb, va);
    float t = fabsf(diff) > 1.0e-8f ? __fdiv_rn(__fsub_rn(g.iso, va), diff) : 0.5f;
    t = t < 0.0f ? 0.0f : (1.0f < t ? 1.0f : t);
    float p[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const float pa = __fadd_rn(g.origin[d], __fmul_rn(static_cast<float>(ca[d]), g.cell[d]));
        const float pb = __fadd_rn(g.origin[d], __fmul_rn(static_cast<float>(cb[d]), g.cell[d]));
        p[d] = __fadd_rn(pa, __fmul_rn(__fsub_rn(pb, pa), t));
    }
    const float3 ga = gradient(field, s, ca[0], ca[1], ca[2], g);
    const float3 gb = gradient(field, s, cb[0], cb[1], cb[2], g);
    // Outward normal: minus the interpolated gradient.
    float nx = -__fadd_rn(ga.x, __fmul_rn(__fsub_rn(gb.x, ga.x), t));
    float ny = -__fadd_rn(ga.y, __fmul_rn(__fsub_rn(gb.y, ga.y), t));
    float nz = -__fadd_rn(ga.z, __fmul_rn(__fsub_rn(gb.z, ga.z), t));
    if (!(__fsqrt_rn(dot3(nx, ny, nz)) > 1.0e-12f)) {
        nx = 0.0f;
        ny = 1.0f;
        nz = 0.0f;
    }
    // glm::normalize: v * (1 / sqrt(dot(v, v))).
    const float inv = __fdiv_rn(1.0f, __fsqrt_rn(dot3(nx, ny, nz)));
    sph_surface_vertex vert;
    vert.position[0] = p[0];
    vert.position[1] = p[1];
    vert.position[2] = p[2];
    vert.normal = pack_unit_vector(__fmul_rn(nx, inv), __fmul_rn(ny, inv), __fmul_rn(nz, inv));
    return vert;
}

// Places every cell's vertices at its serial slot (marching_cubes.cpp:397-481).
// Few cells cut the surface, so the block first lays out its tile (codes and
// each thread's first vertex in shared memory) and then deals the tile's
// vertices out round-robin: a thread finds a vertex's cell by binary search
// over the threads' first vertices and a walk over that thread's cells.
__global__ void __launch_bounds__(kBlock) emit_kernel(const float* __restrict__ field, MarchGeom g,
                                                      const uint8_t* __restrict__ codes,
                                                      const uint32_t* __restrict__ offsets, uint32_t capacity,
                                                      uint32_t* __restrict__ limit,
                                                      sph_surface_vertex* __restrict__ out) {
    __shared__ uint8_t s_code[kTile];
    __shared__ uint32_t s_first[kBlock + 1];
    __shared__ uint32_t total;
    __shared__ alignas(16) int8_t s_entry[256][SPH_MC_TABLE_WIDTH];
    __shared__ uint8_t s_count[256];
    static_assert(kBlock == 256 && SPH_MC_TABLE_WIDTH == 16, "one thread stages one case's row and count");
    reinterpret_cast<uint4*>(&s_entry[0][0])[threadIdx.x] = reinterpret_cast<const uint4*>(&g_entry[0][0])[threadIdx.x];
    s_count[threadIdx.x] = g_count[threadIdx.x];
    __syncthreads();
    const uint32_t cells = g.resolution * g.resolution * g.resolution;
    const uint32_t tile_first = blockIdx.x * kTile;
    uint32_t sum = 0;
#pragma unroll
    for (uint32_t k = 0; k < kPerThread; ++k) {
        const uint32_t cell = tile_first + threadIdx.x * kPerThread + k;
        const uint32_t code = cell < cells ? codes[cell] : 0u;
        s_code[threadIdx.x * kPerThread + k] = static_cast<uint8_t>(code);
        sum += s_count[code];
    }
    s_first[threadIdx.x] = block_exclusive_scan(sum, &total);
    if (threadIdx.x == 0) {
        s_first[kBlock] = total;
    }
    __syncthreads();
    const uint32_t block_slot = offsets[blockIdx.x];
    const uint32_t vertices = s_first[kBlock];
    for (uint32_t v = threadIdx.x; v < vertices; v += kBlock) {
        // The thread whose vertices hold v: the last t with s_first[t] <= v
        // (threads without vertices share their successor's first vertex).
        uint32_t lo = 0;
        uint32_t hi = kBlock;
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (s_first[mid] <= v) {
                lo = mid;
            } else {
                hi = mid;
            }
        }
        uint32_t rem = v - s_first[lo];
        uint32_t local = s_first[lo];
        uint32_t k = lo * kPerThread;
        uint32_t n = s_count[s_code[k]];
        while (rem >= n) {
            rem -= n;
            local += n;
            n = s_count[s_code[++k]];
        }
        const uint32_t slot = block_slot + local;  // the cell's first vertex
        if (slot + n > capacity) {
            // The cell and every later one are dropped, as in the reference.
            atomicMin(limit, slot);
            continue;
        }
        out[slot + rem] = cell_vertex(field, g, tile_first + k, s_entry[s_code[k]], rem);
    }
}

std::mutex g_upload_guard;
uint64_t g_uploaded = 0;  // bit d: device d has the tables

}  // namespace

const int8_t* case_table() { return &tables().entry[0][0]; }

cudaError_t ensure_tables() {
    int device = 0;
    cudaError_t err = cudaGetDevice(&device);
    if (err != cudaSuccess) {
        return err;
    }
    std::lock_guard<std::mutex> lock(g_upload_guard);
    if (device < 64 && (g_uploaded >> device & 1u) != 0) {
        return cudaSuccess;
    }
    const Tables& t = tables();
    if ((err = cudaMemcpyToSymbol(g_entry, t.entry, sizeof(t.entry))) != cudaSuccess ||
        (err = cudaMemcpyToSymbol(g_count, t.count, sizeof(t.count))) != cudaSuccess) {
        return err;
    }
    if (device < 64) {
        g_uploaded |= 1ull << device;
    }
    return cudaSuccess;
}

uint32_t march_tiles(uint32_t resolution) {
    const uint64_t cells = static_cast<uint64_t>(resolution) * resolution * resolution;
    return static_cast<uint32_t>((cells + kTile - 1) / kTile);
}

cudaError_t launch_field(const float4* spos, const uint2* bucket, const FieldGeom& g, FieldRuns* runs, float* field,
                         cudaStream_t stream) {
    const size_t samples = g.resolution + 1ull;
    cudaError_t err = cudaMemsetAsync(field, 0, samples * samples * samples * sizeof(float), stream);
    if (err != cudaSuccess) {
        return err;
    }
    field_runs_kernel<<<3, 1024, 0, stream>>>(g, runs);
    // Lane groups and samples per lane from the box sizes: a cell holds at
    // most floor(radius / cell) + 1 samples along an axis, radius / cell on
    // average.
    float most = 1.0f;
    float mean = 1.0f;
    for (int a = 0; a < 3; ++a) {
        const float per = g.cell[a] > 0.0f ? g.radius / g.cell[a] : 0.0f;
        const float cap = static_cast<float>(g.resolution);
        most *= std::min(std::floor(per) + 1.0f, cap);
        mean *= std::min(std::max(per, 1.0f), cap);
    }
    int device = 0;
    int sms = 0;
    if ((err = cudaGetDevice(&device)) != cudaSuccess ||
        (err = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device)) != cudaSuccess) {
        return err;
    }
    const uint32_t blocks = static_cast<uint32_t>(sms) * 8u;  // grid-stride over the cell boxes
    if (most <= 8.0f) {
        field_cells_kernel<8, 1><<<blocks, kBlock, 0, stream>>>(spos, bucket, g, runs, field);
    } else if (most <= 16.0f || mean <= 12.0f) {
        field_cells_kernel<16, 1><<<blocks, kBlock, 0, stream>>>(spos, bucket, g, runs, field);
    } else if (most <= 32.0f) {
        field_cells_kernel<32, 1><<<blocks, kBlock, 0, stream>>>(spos, bucket, g, runs, field);
    } else if (most <= 64.0f) {
        field_cells_kernel<32, 2><<<blocks, kBlock, 0, stream>>>(spos, bucket, g, runs, field);
    } else {
        field_cells_kernel<32, 4><<<blocks, kBlock, 0, stream>>>(spos, bucket, g, runs, field);
    }
    return cudaGetLastError();
}

cudaError_t launch_march(const float* field, const MarchGeom& g, uint32_t capacity, MarchScratch s,
                         sph_surface_vertex* out, cudaStream_t stream) {
    cudaError_t err = ensure_tables();
    if (err != cudaSuccess) {
        return err;
    }
    const uint32_t tiles = march_tiles(g.resolution);
    if ((err = cudaMemsetAsync(s.limit, 0xFF, sizeof(uint32_t), stream)) != cudaSuccess) {
        return err;
    }
    count_kernel<<<tiles, kBlock, 0, stream>>>(field, g, s.codes, s.tile_sums);
    tile_scan_kernel<<<1, 1024, 0, stream>>>(s.tile_sums, tiles, s.offsets);
    emit_kernel<<<tiles, kBlock, 0, stream>>>(field, g, s.codes, s.offsets, capacity, s.limit, out);
    return cudaGetLastError();
}

}  // namespace surface
}  // namespace sph
