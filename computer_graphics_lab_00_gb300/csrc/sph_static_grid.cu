// sph_static_grid.cu — the grid build (keys, stable radix sort, bucket
// slots) for callers that cannot allocate device memory when they call it.
//
// The sort needs scratch beyond its inputs and outputs: two ping-pong
// (key, id) arrays, the digit histograms and a (start, end) table per bucket.
// Here that scratch is one file-scope device array of a fixed size, so the
// call itself performs no cudaMalloc, cudaFree or other allocation. The array
// belongs to the loaded library: every GPU that uses this entry point holds
// it (about 1.6 MB) until the process exits.
#include <array>
#include <cstdint>
#include <mutex>

#include "../../include/sph_c.h"
#include "sph_kernels.h"

namespace {

constexpr uint32_t kMaxParticles = SPH_STATIC_MAX_PARTICLES;
constexpr uint32_t kMaxCells = SPH_STATIC_MAX_CELLS;
constexpr uint32_t kMaxTiles = (kMaxParticles + sph::kRadixTile - 1) / sph::kRadixTile;
// keys_a, vals_a, keys_b, vals_b | histograms | bucket start | bucket end
constexpr size_t kScratchWords = 4 * static_cast<size_t>(kMaxParticles) +
                                 static_cast<size_t>(kMaxTiles) * sph::kRadixMaxBins + 2 * static_cast<size_t>(kMaxCells);

static __device__ __align__(256) uint32_t g_grid_scratch[kScratchWords];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
std::array<uint32_t*, kMaxDevices> g_scratch_address{};

// The device address of g_grid_scratch in the current context. Host code must
// not hand the symbol itself to a kernel: on the host it names a stand-in,
// not device memory. The address belongs to the context the library's module
// was loaded into, so it is looked up again on every call made outside a
// stream capture (a host-side table lookup once the module is loaded): after
// a cudaDeviceReset, or with another context current, the next such call
// picks the new address up. A call made while `stream` is being captured
// (where a first lookup could load the module) reuses the address that the
// last uncaptured call on this device found, and fails if there was none.
cudaError_t scratch_for_current_device(cudaStream_t stream, uint32_t** out) {
    int device = 0;
    cudaError_t status = cudaGetDevice(&device);
    if (status != cudaSuccess) {
        return status;
    }
    if (device < 0 || device >= kMaxDevices) {
        return cudaErrorInvalidDevice;
    }
    cudaStreamCaptureStatus capture = cudaStreamCaptureStatusNone;
    cudaError_t query = cudaStreamIsCapturing(stream, &capture);
    bool capturing = query != cudaSuccess || capture != cudaStreamCaptureStatusNone;
    if (query != cudaSuccess) {
        cudaGetLastError();  // e.g. the legacy stream while another stream captures
    }
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!capturing) {
        void* address = nullptr;
        status = cudaGetSymbolAddress(&address, g_grid_scratch);
        if (status != cudaSuccess) {
            return status;
        }
        g_scratch_address[device] = static_cast<uint32_t*>(address);
    } else if (g_scratch_address[device] == nullptr) {
        return cudaErrorStreamCaptureUnsupported;
    }
    *out = g_scratch_address[device];
    return cudaSuccess;
}

// spatialHash(spatialCell(p, h), C) of each particle (spatial_hash.h:12-20).
__global__ void static_keys_kernel(const float4* __restrict__ pos, uint32_t n, float h, uint32_t mask,
                                   uint32_t* __restrict__ cell_of) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) {
        return;
    }
    float4 p = pos[i];
    uint32_t cx = static_cast<uint32_t>(sph::cell_coord(p.x, h));
    uint32_t cy = static_cast<uint32_t>(sph::cell_coord(p.y, h));
    uint32_t cz = static_cast<uint32_t>(sph::cell_coord(p.z, h));
    cell_of[i] = sph::spatial_hash(cx, cy, cz, mask);
}

// Start and end of every bucket's run in the sorted order. Only the buckets
// present are written, and only those are read afterwards, so the table
// needs no clearing between calls.
__global__ void static_bounds_kernel(const uint32_t* __restrict__ sorted_keys, uint32_t n,
                                     uint32_t* __restrict__ start, uint32_t* __restrict__ end) {
    uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) {
        return;
    }
    uint32_t key = sorted_keys[p];
    if (p == 0 || sorted_keys[p - 1] != key) {
        start[key] = p;
    }
    if (p + 1 == n || sorted_keys[p + 1] != key) {
        end[key] = p + 1;
    }
}

// The reference's cellCounts (un-truncated) and cellParticles (first 32 ids
// of each bucket, ascending) (fluid_sph.cpp:181-187).
__global__ void static_slots_kernel(const uint32_t* __restrict__ sorted_keys, const uint32_t* __restrict__ sorted_ids,
                                    uint32_t n, const uint32_t* __restrict__ start, const uint32_t* __restrict__ end,
                                    uint32_t* __restrict__ cell_counts, uint32_t* __restrict__ cell_particles) {
    uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) {
        return;
    }
    uint32_t key = sorted_keys[p];
    uint32_t first = start[key];
    uint32_t slot = p - first;
    if (slot < sph::kCellCapacity) {
        cell_particles[static_cast<size_t>(key) * sph::kCellCapacity + slot] = sorted_ids[p];
    }
    if (slot == 0) {
        cell_counts[key] = end[key] - first;
    }
}

uint32_t bit_width(uint32_t v) {
    uint32_t bits = 0;
    while (v != 0) {
        ++bits;
        v >>= 1;
    }
    return bits;
}

}  // namespace

extern "C" int sph_grid_build_static(const sph_params* params,
                                     const void* positions,
                                     uint32_t count,
                                     void* cell_of,
                                     void* cell_counts,
                                     void* cell_particles,
                                     void* stream) {
    if (params == nullptr) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    uint32_t cells = params->lattice[3];
    float h = params->smoothing_radius;
    if (cells == 0 || (cells & (cells - 1)) != 0 || !(h > 0.0F)) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    if (count > kMaxParticles || cells > kMaxCells) {
        return SPH_ERR_CAPACITY;
    }
    if (cell_counts == nullptr || (count > 0 && (positions == nullptr || cell_of == nullptr)) ||
        cell_particles == nullptr) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    // Positions are read as float4 (16-byte loads); the u32 arrays as words.
    auto misaligned = [](const void* p, uintptr_t a) { return (reinterpret_cast<uintptr_t>(p) % a) != 0; };
    if (misaligned(positions, 16) || misaligned(cell_of, 4) || misaligned(cell_counts, 4) ||
        misaligned(cell_particles, 4)) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // This library's CUDA runtime is private to it, so an error pending in it
    // was left by an earlier call of this library; it is not this call's.
    cudaGetLastError();
    uint32_t* scratch = nullptr;
    if (scratch_for_current_device(s, &scratch) != cudaSuccess) {
        cudaGetLastError();
        return SPH_ERR_CUDA;
    }
    auto* counts = static_cast<uint32_t*>(cell_counts);
    if (cudaMemsetAsync(counts, 0, sizeof(uint32_t) * cells, s) != cudaSuccess) {
        cudaGetLastError();
        return SPH_ERR_CUDA;
    }
    if (count == 0) {
        return SPH_OK;
    }
    auto* keys = static_cast<uint32_t*>(cell_of);
    static_keys_kernel<<<(count + 255) / 256, 256, 0, s>>>(static_cast<const float4*>(positions), count, h, cells - 1U,
                                                          keys);
    if (cudaGetLastError() != cudaSuccess) {
        return SPH_ERR_CUDA;
    }
    sph::GridScratch grid;
    grid.keys = keys;
    grid.keys_a = scratch;
    grid.vals_a = scratch + kMaxParticles;
    grid.keys_b = scratch + 2 * static_cast<size_t>(kMaxParticles);
    grid.vals_b = scratch + 3 * static_cast<size_t>(kMaxParticles);
    grid.hist = scratch + 4 * static_cast<size_t>(kMaxParticles);
    uint32_t* start = grid.hist + static_cast<size_t>(kMaxTiles) * sph::kRadixMaxBins;
    uint32_t* end = start + kMaxCells;
    sph::RadixPlan plan = sph::plan_radix(bit_width(cells - 1U), 6);
    if (sph::launch_radix_sort(grid, count, plan, s, nullptr) != cudaSuccess) {
        cudaGetLastError();
        return SPH_ERR_CUDA;
    }
    static_bounds_kernel<<<(count + 255) / 256, 256, 0, s>>>(grid.sorted_keys, count, start, end);
    if (cudaGetLastError() != cudaSuccess) {
        return SPH_ERR_CUDA;
    }
    static_slots_kernel<<<(count + 255) / 256, 256, 0, s>>>(grid.sorted_keys, grid.sorted_ids, count, start, end,
                                                           counts, static_cast<uint32_t*>(cell_particles));
    if (cudaGetLastError() != cudaSuccess) {
        return SPH_ERR_CUDA;
    }
    return SPH_OK;
}
