// sph_grid.cu — spatial-hash grid build on the GPU.
//
// The reference inserts particles serially in ascending id into fixed
// 32-slot buckets (src/physics/fluid_sph.cpp:160-188) so that every bucket
// lists its particles in id order, and its Vulkan twin does the same insert
// with one atomic per particle (shaders/fluid_grid.comp:9-21), which loses
// that order. Here the grid is a stable counting sort instead: keys are
// bucket indices, an LSD radix sort over (key, id) keeps ids ascending inside
// every bucket, and a bounds pass turns the sorted keys into a
// (start, end) table. The first min(count, 32) ids of a bucket are exactly
// the reference's cellParticles slots and end - start is its un-truncated
// cellCounts entry.
//
// Digit histograms use warp-aggregated shared-memory atomics
// (__match_any_sync groups lanes with the same digit; one lane adds the
// group's population). Ranks inside a tile come from the same match masks,
// so the sort is stable without any per-element atomics in global memory.
#include "sph_kernels.h"

#include <cstring>

namespace sph {

namespace {

__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t mask;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(mask));
    return mask;
}

__global__ void __launch_bounds__(256) keys_kernel(const float4* __restrict__ pos, const uint16_t* __restrict__ tank_of,
                                                   const TankConst* __restrict__ tanks, uint32_t n,
                                                   uint32_t* __restrict__ keys) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) {
        return;
    }
    const TankConst* t = tanks + (tank_of != nullptr ? tank_of[i] : 0);
    float h = __ldg(&t->h);
    float4 p = pos[i];
    uint32_t cx = static_cast<uint32_t>(cell_coord(p.x, h));
    uint32_t cy = static_cast<uint32_t>(cell_coord(p.y, h));
    uint32_t cz = static_cast<uint32_t>(cell_coord(p.z, h));
    keys[i] = __ldg(&t->bucket_base) + spatial_hash(cx, cy, cz, __ldg(&t->cell_mask));
}

// ---- counting placement (grid sort mode 2) -----------------------------------
//
// The grid without a radix sort. Every particle takes a place in its bucket
// with one atomic add (count_keys_kernel), an exclusive scan of the bucket
// counts gives every bucket its range in the sorted arrays (and so the bucket
// table), and the particles are placed in those ranges in the atomics'
// arbitrary order (place_kernel). order_gather_kernel then puts each bucket's
// first min(count, 32) particles by id at the front of its range in ascending
// id order, which is the reference's insertion order (fluid_sph.cpp:160-188),
// and gathers their state there; the rest of an overflowing bucket follows in
// any order, and no neighbour walk reads past its 32nd entry.

constexpr uint32_t kScanItems = 4;                        // counts per thread of a scan block
constexpr uint32_t kScanTile = 256 * kScanItems;          // 1,024 buckets per scan block (more blocks in flight)

__global__ void __launch_bounds__(256) count_keys_kernel(const float4* __restrict__ pos,
                                                         const uint16_t* __restrict__ tank_of,
                                                         const TankConst* __restrict__ tanks, uint32_t n,
                                                         uint32_t* __restrict__ keys, uint32_t* __restrict__ ranks,
                                                         uint32_t* __restrict__ counts) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) {
        return;
    }
    const TankConst* t = tanks + (tank_of != nullptr ? tank_of[i] : 0);
    const float h = __ldg(&t->h);
    const float4 p = pos[i];
    const uint32_t cx = static_cast<uint32_t>(cell_coord(p.x, h));
    const uint32_t cy = static_cast<uint32_t>(cell_coord(p.y, h));
    const uint32_t cz = static_cast<uint32_t>(cell_coord(p.z, h));
    const uint32_t key = __ldg(&t->bucket_base) + spatial_hash(cx, cy, cz, __ldg(&t->cell_mask));
    keys[i] = key;
    ranks[i] = atomicAdd(&counts[key], 1u);
}

// Block sums of the bucket counts, kScanTile buckets a block.
__global__ void __launch_bounds__(256) scan_reduce_kernel(const uint32_t* __restrict__ counts, uint32_t buckets,
                                                          uint32_t* __restrict__ block_sums) {
    const uint32_t first = blockIdx.x * kScanTile;
    uint32_t sum = 0;
#pragma unroll
    for (uint32_t r = 0; r < kScanItems; ++r) {
        const uint32_t b = first + r * 256u + threadIdx.x;
        sum += b < buckets ? __ldg(&counts[b]) : 0u;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        sum += __shfl_down_sync(0xFFFFFFFFu, sum, o);
    }
    __shared__ uint32_t warp_sums[8];
    if ((threadIdx.x & 31u) == 0) {
        warp_sums[threadIdx.x >> 5] = sum;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t total = 0;
#pragma unroll
        for (int w = 0; w < 8; ++w) {
            total += warp_sums[w];
        }
        block_sums[blockIdx.x] = total;
    }
}

// Exclusive scan of the block sums in place: one block of 1,024 threads, in
// rounds of 1,024 sums carried over.
__global__ void __launch_bounds__(1024) scan_top_kernel(uint32_t* __restrict__ block_sums, uint32_t blocks) {
    __shared__ uint32_t warp_sums[32];
    __shared__ uint32_t carry;
    if (threadIdx.x == 0) {
        carry = 0;
    }
    __syncthreads();
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t warp = threadIdx.x >> 5;
    for (uint32_t base = 0; base < blocks; base += 1024u) {
        const uint32_t b = base + threadIdx.x;
        const uint32_t v = b < blocks ? block_sums[b] : 0u;
        uint32_t inc = v;
#pragma unroll
        for (uint32_t o = 1; o < 32u; o <<= 1) {
            const uint32_t u = __shfl_up_sync(0xFFFFFFFFu, inc, o);
            if (lane >= o) {
                inc += u;
            }
        }
        if (lane == 31u) {
            warp_sums[warp] = inc;
        }
        __syncthreads();
        if (warp == 0) {
            uint32_t w = warp_sums[lane];
            uint32_t winc = w;
#pragma unroll
            for (uint32_t o = 1; o < 32u; o <<= 1) {
                const uint32_t u = __shfl_up_sync(0xFFFFFFFFu, winc, o);
                if (lane >= o) {
                    winc += u;
                }
            }
            warp_sums[lane] = winc - w;  // exclusive warp offsets
        }
        __syncthreads();
        const uint32_t before = carry + warp_sums[warp] + inc - v;
        if (b < blocks) {
            block_sums[b] = before;
        }
        __syncthreads();
        if (threadIdx.x == 1023u) {
            carry = before + v;
        }
        __syncthreads();
    }
}

// The bucket table from the counts and the scanned block sums: bucket b's
// range is [start, start + count) in the sorted arrays. The counts are reset
// on the way (the final ordering counts an overflowing bucket's tail in them).
__global__ void __launch_bounds__(256) scan_down_kernel(uint32_t* __restrict__ counts, uint32_t buckets,
                                                        const uint32_t* __restrict__ block_sums,
                                                        uint2* __restrict__ bucket) {
    static_assert(kScanItems % 4 == 0, "counts move as uint4");
    const uint32_t first = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    uint32_t c[kScanItems];
    // Whole uint4 groups when the thread's buckets are all present (buckets
    // is then a multiple of 4 past them); element by element at the end.
    const bool whole = first + kScanItems <= buckets;
    if (whole) {
        const uint4* src = reinterpret_cast<const uint4*>(counts + first);
#pragma unroll
        for (uint32_t r = 0; r < kScanItems / 4; ++r) {
            const uint4 v = src[r];
            c[4 * r] = v.x;
            c[4 * r + 1] = v.y;
            c[4 * r + 2] = v.z;
            c[4 * r + 3] = v.w;
        }
    } else {
#pragma unroll
        for (uint32_t r = 0; r < kScanItems; ++r) {
            c[r] = first + r < buckets ? counts[first + r] : 0u;
        }
    }
    uint32_t sum = 0;
#pragma unroll
    for (uint32_t r = 0; r < kScanItems; ++r) {
        sum += c[r];
    }
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t warp = threadIdx.x >> 5;
    uint32_t inc = sum;
#pragma unroll
    for (uint32_t o = 1; o < 32u; o <<= 1) {
        const uint32_t u = __shfl_up_sync(0xFFFFFFFFu, inc, o);
        if (lane >= o) {
            inc += u;
        }
    }
    __shared__ uint32_t warp_sums[8];
    if (lane == 31u) {
        warp_sums[warp] = inc;
    }
    __syncthreads();
    uint32_t start = block_sums[blockIdx.x] + inc - sum;
    for (uint32_t w = 0; w < warp; ++w) {
        start += warp_sums[w];
    }
    if (whole) {
        uint4* dst = reinterpret_cast<uint4*>(bucket + first);
#pragma unroll
        for (uint32_t r = 0; r < kScanItems / 2; ++r) {
            const uint32_t a = start;
            const uint32_t b = a + c[2 * r];
            const uint32_t e = b + c[2 * r + 1];
            dst[r] = make_uint4(a, b, b, e);
            start = e;
        }
        uint4* zero = reinterpret_cast<uint4*>(counts + first);
#pragma unroll
        for (uint32_t r = 0; r < kScanItems / 4; ++r) {
            zero[r] = make_uint4(0u, 0u, 0u, 0u);
        }
    } else {
#pragma unroll
        for (uint32_t r = 0; r < kScanItems; ++r) {
            const uint32_t b = first + r;
            if (b < buckets) {
                bucket[b] = make_uint2(start, start + c[r]);
                counts[b] = 0;
            }
            start += c[r];
        }
    }
}

// Each particle at its bucket's start plus its atomic rank (any order).
__global__ void __launch_bounds__(256) place_kernel(const uint32_t* __restrict__ keys,
                                                    const uint32_t* __restrict__ ranks, uint32_t n,
                                                    const uint2* __restrict__ bucket, uint32_t* __restrict__ placed) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        placed[__ldg(&bucket[keys[i]]).x + ranks[i]] = i;
    }
}

// The final order and the gather in one pass, a thread per placed slot:
// particle i (placed in its bucket in the atomics' order) counts the members
// of its bucket with a smaller id (all of them in a bucket of at most
// kCountAll, else until it has found 32), which is its place when below 32
// (the reference's insertion order, ascending ids); the rest of an
// overflowing bucket follows the 32 in any order (an atomic count), and no
// neighbour walk reads past a bucket's 32nd entry. The particle's state, tank
// and processing slot go to that place as bounds_gather_kernel writes them.
constexpr uint32_t kCountAll = 64;  // buckets up to this size are ranked in full

__global__ void __launch_bounds__(256) order_gather_kernel(const uint32_t* __restrict__ keys,
                                                           const uint32_t* __restrict__ placed, uint32_t n,
                                                           const uint2* __restrict__ bucket,
                                                           uint32_t* __restrict__ tail_counts,
                                                           uint32_t* __restrict__ sorted_ids,
                                                           const float4* __restrict__ pos,
                                                           const float4* __restrict__ vel,
                                                           const uint16_t* __restrict__ tank_of,
                                                           float4* __restrict__ spos, float4* __restrict__ svel,
                                                           uint16_t* __restrict__ stank, Schedule schedule) {
    const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) {
        return;
    }
    const uint32_t i = placed[q];
    const uint32_t key = keys[i];
    const uint2 r = __ldg(&bucket[key]);
    const bool full = r.y - r.x <= kCountAll;
    uint32_t smaller = 0;
    for (uint32_t k = r.x; k < r.y && (full || smaller < kCellCapacity); ++k) {
        smaller += __ldg(&placed[k]) < i ? 1u : 0u;
    }
    const uint32_t p = full || smaller < kCellCapacity ? r.x + smaller
                                                        : r.x + kCellCapacity + atomicAdd(&tail_counts[key], 1u);
    sorted_ids[p] = i;
    spos[p] = pos[i];
    if (vel != nullptr) {  // else gather_vel_kernel writes them later
        svel[p] = vel[i];
    }
    if (tank_of != nullptr) {
        stank[p] = tank_of[i];
    }
    if (schedule.rank != nullptr) {
        schedule.order[schedule.rank[i]] = p;
    }
}

// Per-tile digit histogram, written digit-major: hist[d * tiles + tile].
__global__ void __launch_bounds__(kRadixThreads) radix_upsweep(const uint32_t* __restrict__ keys, uint32_t n,
                                                               uint32_t shift, uint32_t mask, uint32_t tiles,
                                                               uint32_t* __restrict__ hist) {
    __shared__ uint32_t counts[kRadixMaxBins];
    for (uint32_t d = threadIdx.x; d <= mask; d += blockDim.x) {
        counts[d] = 0;
    }
    __syncthreads();
    uint32_t warp = threadIdx.x >> 5;
    uint32_t lane = threadIdx.x & 31;
    uint32_t base = blockIdx.x * kRadixTile + warp * (kRadixItems * 32);
#pragma unroll 4
    for (uint32_t r = 0; r < kRadixItems; ++r) {
        uint32_t idx = base + r * 32 + lane;
        bool valid = idx < n;
        uint32_t digit = valid ? (keys[idx] >> shift) & mask : 0xFFFFFFFFu;
        uint32_t peers = __match_any_sync(0xFFFFFFFFu, digit);
        if (valid && lane == static_cast<uint32_t>(__ffs(peers) - 1)) {
            atomicAdd(&counts[digit], static_cast<uint32_t>(__popc(peers)));
        }
    }
    __syncthreads();
    for (uint32_t d = threadIdx.x; d <= mask; d += blockDim.x) {
        hist[d * tiles + blockIdx.x] = counts[d];
    }
}

// Exclusive scan of m counters in one block of 1024 threads (m is bins x
// tiles, at most a few hundred thousand). Each pass scans 8192 counters:
// every thread loads 8 consecutive ones (a warp reads 1 KB contiguous), the
// thread totals are scanned across the block, and a carry links the passes.
__global__ void __launch_bounds__(1024) scan_exclusive_block(uint32_t* __restrict__ data, uint32_t m) {
    __shared__ uint32_t warp_sums[32];
    __shared__ uint32_t block_total;
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t warp = threadIdx.x >> 5;
    uint32_t carry = 0;
    for (uint32_t base = 0; base < m; base += 8 * 1024) {
        uint32_t first = base + threadIdx.x * 8;
        uint32_t v[8];
        uint32_t local = 0;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            v[k] = first + k < m ? data[first + k] : 0;
            local += v[k];
        }
        uint32_t inclusive = local;
#pragma unroll
        for (uint32_t o = 1; o < 32; o <<= 1) {
            uint32_t u = __shfl_up_sync(0xFFFFFFFFu, inclusive, o);
            if (lane >= o) {
                inclusive += u;
            }
        }
        if (lane == 31) {
            warp_sums[warp] = inclusive;
        }
        __syncthreads();
        if (warp == 0) {
            uint32_t w = warp_sums[lane];
            uint32_t inc = w;
#pragma unroll
            for (uint32_t o = 1; o < 32; o <<= 1) {
                uint32_t u = __shfl_up_sync(0xFFFFFFFFu, inc, o);
                if (lane >= o) {
                    inc += u;
                }
            }
            warp_sums[lane] = inc - w;
            if (lane == 31) {
                block_total = inc;
            }
        }
        __syncthreads();
        uint32_t run = carry + warp_sums[warp] + inclusive - local;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            if (first + k < m) {
                data[first + k] = run;
            }
            run += v[k];
        }
        carry += block_total;
        __syncthreads();
    }
}

// Stable scatter of one radix pass. Warp w of a tile owns 512 consecutive
// keys and walks them in 16 rounds of 32, so (round, lane) is input order;
// the per-warp digit counters give each key its rank among equal digits
// before it, and a prefix over warps makes the rank tile-wide.
__global__ void __launch_bounds__(kRadixThreads) radix_downsweep(const uint32_t* __restrict__ keys_in,
                                                                 const uint32_t* __restrict__ vals_in,
                                                                 uint32_t* __restrict__ keys_out,
                                                                 uint32_t* __restrict__ vals_out, uint32_t n,
                                                                 uint32_t shift, uint32_t mask, uint32_t tiles,
                                                                 const uint32_t* __restrict__ hist) {
    constexpr uint32_t kWarps = kRadixThreads / 32;
    __shared__ uint32_t warp_counts[kWarps][kRadixMaxBins];
    __shared__ uint32_t tile_offset[kRadixMaxBins];
    for (uint32_t k = threadIdx.x; k < kWarps * kRadixMaxBins; k += blockDim.x) {
        (&warp_counts[0][0])[k] = 0;
    }
    __syncthreads();
    uint32_t warp = threadIdx.x >> 5;
    uint32_t lane = threadIdx.x & 31;
    uint32_t below = lanemask_lt();
    uint32_t base = blockIdx.x * kRadixTile + warp * (kRadixItems * 32);
    uint32_t key[kRadixItems];
    uint32_t val[kRadixItems];
    uint32_t rank[kRadixItems];
#pragma unroll
    for (uint32_t r = 0; r < kRadixItems; ++r) {
        uint32_t idx = base + r * 32 + lane;
        bool valid = idx < n;
        key[r] = valid ? keys_in[idx] : 0;
        val[r] = valid ? (vals_in != nullptr ? vals_in[idx] : idx) : 0;
        uint32_t digit = valid ? (key[r] >> shift) & mask : 0xFFFFFFFFu;
        uint32_t peers = __match_any_sync(0xFFFFFFFFu, digit);
        uint32_t before = valid ? warp_counts[warp][digit] : 0;
        rank[r] = valid ? before + static_cast<uint32_t>(__popc(peers & below)) : 0xFFFFFFFFu;
        __syncwarp();
        if (valid && lane == static_cast<uint32_t>(__ffs(peers) - 1)) {
            warp_counts[warp][digit] = before + static_cast<uint32_t>(__popc(peers));
        }
        __syncwarp();
    }
    __syncthreads();
    for (uint32_t d = threadIdx.x; d <= mask; d += blockDim.x) {
        uint32_t running = 0;
#pragma unroll
        for (uint32_t w = 0; w < kWarps; ++w) {
            uint32_t c = warp_counts[w][d];
            warp_counts[w][d] = running;
            running += c;
        }
        tile_offset[d] = hist[d * tiles + blockIdx.x];
    }
    __syncthreads();
#pragma unroll
    for (uint32_t r = 0; r < kRadixItems; ++r) {
        if (rank[r] != 0xFFFFFFFFu) {
            uint32_t digit = (key[r] >> shift) & mask;
            uint32_t dst = tile_offset[digit] + warp_counts[warp][digit] + rank[r];
            keys_out[dst] = key[r];
            vals_out[dst] = val[r];
        }
    }
}

__device__ __forceinline__ uint32_t spread3(uint32_t v) {
    v &= 0x3FFu;
    v = (v | (v << 16)) & 0x030000FFu;
    v = (v | (v << 8)) & 0x0300F00Fu;
    v = (v | (v << 4)) & 0x030C30C3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

__global__ void __launch_bounds__(256) bounds_gather_kernel(const uint32_t* __restrict__ sorted_keys,
                                                            const uint32_t* __restrict__ sorted_ids, uint32_t n,
                                                            uint32_t* __restrict__ bucket_words,
                                                            const float4* __restrict__ pos,
                                                            const float4* __restrict__ vel,
                                                            const uint16_t* __restrict__ tank_of,
                                                            float4* __restrict__ spos, float4* __restrict__ svel,
                                                            uint16_t* __restrict__ stank, Schedule schedule,
                                                            const uint32_t* __restrict__ ids,
                                                            uint32_t* __restrict__ global_sorted) {
    uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) {
        return;
    }
    if (sorted_keys != nullptr) {  // else the counting placement wrote the bucket table
        uint32_t key = sorted_keys[p];
        if (p == 0 || sorted_keys[p - 1] != key) {
            bucket_words[2 * static_cast<size_t>(key)] = p;
        }
        if (p + 1 == n || sorted_keys[p + 1] != key) {
            bucket_words[2 * static_cast<size_t>(key) + 1] = p + 1;
        }
    }
    uint32_t i = sorted_ids[p];
    if (ids != nullptr) {
        // A compacted particle set: sorted entries are positions in `ids`.
        i = ids[i];
        global_sorted[p] = i;
    }
    spos[p] = pos[i];
    if (vel != nullptr) {  // else gather_vel_kernel writes them later
        svel[p] = vel[i];
    }
    if (tank_of != nullptr) {
        stank[p] = tank_of[i];
    }
    if (schedule.rank != nullptr) {
        schedule.order[schedule.rank[i]] = p;
    }
}

// The velocities of a gather that skipped them: svel[p].xyz = vel[i].xyz,
// with no write to .w (the density pass writes the pressure there, and may
// run at the same time).
__global__ void __launch_bounds__(256) gather_vel_kernel(const uint32_t* __restrict__ sorted_ids, uint32_t n,
                                                         const float4* __restrict__ vel, float4* __restrict__ svel) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) {
        return;
    }
    const float4 v = vel[sorted_ids[p]];
    float* row = reinterpret_cast<float*>(svel + p);
    *reinterpret_cast<float2*>(row) = make_float2(v.x, v.y);
    row[2] = v.z;
}

// Processing slot of every particle id: the inverse of the Morton-sorted ids
// (entries of a compacted set name ids[entry]).
__global__ void __launch_bounds__(256) rank_kernel(const uint32_t* __restrict__ sorted_ids, uint32_t n,
                                                   uint32_t* __restrict__ rank, const uint32_t* __restrict__ ids) {
    uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) {
        const uint32_t v = sorted_ids[t];
        rank[ids != nullptr ? ids[v] : v] = t;
    }
}

// ---- one kernel per digit pass -----------------------------------------------------
//
// Each pass knows, before it starts, how many keys of every digit each tile
// holds (tile_counts, tiles x bins): the key kernel counts the first pass's
// tiles, and every pass counts the next pass's tiles while it scatters. A
// tile's offset for digit d is then the digit's base (exclusive scan of the
// pass histogram) plus the sum of d's counts over the earlier tiles, which
// each block adds up on its own: no block waits on another.

// Above kChunkedTiles tiles a pass block would sum too many earlier tiles'
// digit counts (the work grows with the square of the tile count), so a small
// kernel first sums each chunk of kChunkTiles tiles, and a block then adds
// the whole chunks before its own and the tiles of its own chunk.
constexpr uint32_t kChunkTiles = 32;
constexpr uint32_t kChunkedTiles = 256;

inline uint32_t sweep_chunks(uint32_t tiles) { return (tiles + kChunkTiles - 1) / kChunkTiles; }

struct SweepLayout {
    uint32_t* tile_counts;  // passes x tiles x bins
    uint32_t* hist;         // passes x bins
    uint32_t* chunk_sums;   // chunks x bins (one pass at a time)
};

__host__ __device__ inline SweepLayout sweep_layout(unsigned long long* base, uint32_t tiles, uint32_t passes) {
    SweepLayout l;
    l.tile_counts = reinterpret_cast<uint32_t*>(base);
    l.hist = l.tile_counts + static_cast<size_t>(passes) * tiles * kSweepBins;
    l.chunk_sums = l.hist + static_cast<size_t>(passes) * kSweepBins;
    return l;
}

// chunk_sums[c][d] = the digit-d counts of tiles 32c .. 32c + 31 (one block a
// chunk, one thread a digit).
__global__ void __launch_bounds__(kSweepBins) chunk_sums_kernel(const uint32_t* __restrict__ tile_counts,
                                                                uint32_t tiles, uint32_t* __restrict__ chunk_sums) {
    const uint32_t c = blockIdx.x;
    const uint32_t d = threadIdx.x;
    const uint32_t first = c * kChunkTiles;
    const uint32_t last = min(first + kChunkTiles, tiles);
    uint32_t sum = 0;
#pragma unroll 8
    for (uint32_t t = first; t < last; ++t) {
        sum += __ldg(&tile_counts[static_cast<size_t>(t) * kSweepBins + d]);
    }
    chunk_sums[static_cast<size_t>(c) * kSweepBins + d] = sum;
}

// keys_kernel for one tile of kSweepTile particles (1024 threads, four
// particles each, their loads issued together), plus the first pass's tile
// counts and every pass's digit histogram.
constexpr uint32_t kKeysThreads = 1024;
constexpr uint32_t kKeysItems = kSweepTile / kKeysThreads;

// Hilbert index of the cell (x0, x1, x2) of a 2^bits cube, after J.
// Skilling, "Programming the Hilbert curve", AIP Conf. Proc. 707 (2004):
// the coordinates are turned into the curve's "transpose" (undo the
// excess work level by level, then Gray-code), whose bits, interleaved with
// x0's bit highest at each level, are the index. Consecutive indices are
// face-adjacent cells, so runs of the order stay compact at every scale.
__device__ __forceinline__ uint32_t hilbert3(uint32_t x0, uint32_t x1, uint32_t x2, uint32_t bits) {
    uint32_t x[3] = {x0, x1, x2};
    const uint32_t top = 1u << (bits - 1u);
    for (uint32_t q = top; q > 1u; q >>= 1) {
        const uint32_t low = q - 1u;
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            if (x[i] & q) {
                x[0] ^= low;
            } else {
                const uint32_t swap = (x[0] ^ x[i]) & low;
                x[0] ^= swap;
                x[i] ^= swap;
            }
        }
    }
    x[1] ^= x[0];
    x[2] ^= x[1];
    uint32_t flip = 0;
    for (uint32_t q = top; q > 1u; q >>= 1) {
        if (x[2] & q) {
            flip ^= q - 1u;
        }
    }
    return (spread3(x[0] ^ flip) << 2) | (spread3(x[1] ^ flip) << 1) | spread3(x[2] ^ flip);
}

// Curve key of a particle's cell for the processing order: the grid's own
// cell (so a cell's particles stay together), offset from the cell of the
// tank's low corner and clamped to `bits` bits per axis, as a Morton code or
// a Hilbert index, the tank index above it.
__device__ __forceinline__ uint32_t morton_key(float4 p, const TankConst* t, uint32_t tank, uint32_t bits,
                                               bool hilbert) {
    const float h = __ldg(&t->h);
    const int limit = static_cast<int>((1u << bits) - 1u);
    const int cx = min(max(cell_coord(p.x, h) - cell_coord(__ldg(&t->low[0]), h), 0), limit);
    const int cy = min(max(cell_coord(p.y, h) - cell_coord(__ldg(&t->low[1]), h), 0), limit);
    const int cz = min(max(cell_coord(p.z, h) - cell_coord(__ldg(&t->low[2]), h), 0), limit);
    const uint32_t code = hilbert ? hilbert3(static_cast<uint32_t>(cx), static_cast<uint32_t>(cy),
                                             static_cast<uint32_t>(cz), bits)
                                  : spread3(static_cast<uint32_t>(cx)) | (spread3(static_cast<uint32_t>(cy)) << 1) |
                                        (spread3(static_cast<uint32_t>(cz)) << 2);
    return (tank << (3 * bits)) | code;
}

// kMorton false: the spatial-hash bucket keys of the grid (spread evenly over
// the digits); true: Morton keys of the processing order, whose high digits
// bunch up, so the lanes of a warp with the same digit add their counts with
// one atomic.
template <bool kMorton>
__global__ void __launch_bounds__(kKeysThreads) keys_hist_kernel(const float4* __restrict__ pos,
                                                                 const uint16_t* __restrict__ tank_of,
                                                                 const TankConst* __restrict__ tanks, uint32_t n,
                                                                 uint32_t* __restrict__ keys, uint32_t passes,
                                                                 uint32_t* __restrict__ tile_counts,
                                                                 uint32_t* __restrict__ hist, uint32_t morton_bits,
                                                                 const uint32_t* __restrict__ ids, int hilbert,
                                                                 IdSplit split, uint32_t split_at) {
    __shared__ uint32_t counts[kSweepMaxPasses][kSweepBins];
    for (uint32_t k = threadIdx.x; k < kSweepMaxPasses * kSweepBins; k += blockDim.x) {
        (&counts[0][0])[k] = 0;
    }
    const uint32_t first = blockIdx.x * kSweepTile;
    float4 p[kKeysItems];
    uint32_t tank[kKeysItems];
#pragma unroll
    for (uint32_t r = 0; r < kKeysItems; ++r) {
        const uint32_t i = first + r * kKeysThreads + threadIdx.x;
        const uint32_t g = i < n && ids != nullptr ? ids[i] : i;
        p[r] = i < n ? pos[g] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        tank[r] = tank_of != nullptr && i < n ? tank_of[g] : 0;
    }
    __syncthreads();
#pragma unroll
    for (uint32_t r = 0; r < kKeysItems; ++r) {
        const uint32_t i = first + r * kKeysThreads + threadIdx.x;
        const TankConst* t = tanks + tank[r];
        if (kMorton) {
            uint32_t key = morton_key(p[r], t, tank[r], morton_bits, hilbert != 0);
            if (split.count > 1 && i < n) {  // the particle's id range above the curve key
                const uint32_t id = ids != nullptr ? ids[i] : i;
                uint32_t range = 0;
                for (uint32_t c = 1; c < split.count; ++c) {
                    range += id >= split.start[c] ? 1u : 0u;
                }
                key |= range << split_at;
            }
            if (i < n) {
                keys[i] = key;
            }
            for (uint32_t pass = 0; pass < passes; ++pass) {
                const uint32_t digit = i < n ? (key >> (pass * kSweepBits)) & (kSweepBins - 1) : 0xFFFFFFFFu;
                const uint32_t peers = __match_any_sync(0xFFFFFFFFu, digit);
                if (i < n && (threadIdx.x & 31) == static_cast<uint32_t>(__ffs(peers) - 1)) {
                    atomicAdd(&counts[pass][digit], static_cast<uint32_t>(__popc(peers)));
                }
            }
        } else if (i < n) {
            const float h = __ldg(&t->h);
            uint32_t cx = static_cast<uint32_t>(cell_coord(p[r].x, h));
            uint32_t cy = static_cast<uint32_t>(cell_coord(p[r].y, h));
            uint32_t cz = static_cast<uint32_t>(cell_coord(p[r].z, h));
            const uint32_t key = __ldg(&t->bucket_base) + spatial_hash(cx, cy, cz, __ldg(&t->cell_mask));
            keys[i] = key;
            for (uint32_t pass = 0; pass < passes; ++pass) {
                atomicAdd(&counts[pass][(key >> (pass * kSweepBits)) & (kSweepBins - 1)], 1u);
            }
        }
    }
    __syncthreads();
    for (uint32_t d = threadIdx.x; d < kSweepBins; d += blockDim.x) {
        tile_counts[static_cast<size_t>(blockIdx.x) * kSweepBins + d] = counts[0][d];
    }
    for (uint32_t k = threadIdx.x; k < passes * kSweepBins; k += blockDim.x) {
        uint32_t c = (&counts[0][0])[k];
        if (c != 0) {
            atomicAdd(&hist[k], c);
        }
    }
}

// One stable digit pass over tile blockIdx.x. kAggregate: the lanes of a warp
// that add to the same next-pass tile count add once (keys whose digits bunch
// up); otherwise every key adds its own 1 (keys spread evenly).
template <bool kAggregate>
__global__ void __launch_bounds__(kSweepThreads) sweep_scatter_kernel(
    const uint32_t* __restrict__ keys_in, const uint32_t* __restrict__ vals_in, uint32_t* __restrict__ keys_out,
    uint32_t* __restrict__ vals_out, uint32_t n, uint32_t shift, const uint32_t* __restrict__ hist,
    const uint32_t* __restrict__ tile_counts, uint32_t* __restrict__ next_counts, uint32_t next_shift,
    const uint32_t* __restrict__ chunk_sums) {
    static_assert(kSweepThreads % kSweepBins == 0 && kSweepThreads >= kSweepBins,
                  "the first kSweepBins threads each own one digit");
    constexpr uint32_t kWarps = kSweepThreads / 32;
    constexpr uint32_t kRowLanes = kSweepThreads / (kSweepBins / 4);  // count rows read side by side
    __shared__ uint32_t warp_counts[kWarps][kSweepBins];
    __shared__ uint32_t digit_offset[kSweepBins];
    __shared__ uint32_t scan_warp[kSweepBins / 32];
    for (uint32_t k = threadIdx.x; k < kWarps * kSweepBins; k += blockDim.x) {
        (&warp_counts[0][0])[k] = 0;
    }
    const uint32_t tile = blockIdx.x;
    const uint32_t d = threadIdx.x;  // the digit this thread owns (threads below kSweepBins)
    const bool owns_digit = d < kSweepBins;
    const uint32_t warp = threadIdx.x >> 5;
    const uint32_t lane = threadIdx.x & 31;
    // Every digit's keys in all earlier tiles: the block reads the earlier
    // tiles' count rows kRowLanes at a time (a row is 64 uint4, thread k reads
    // column k % 64 of row j + k / 64), eight rows' loads in flight per thread,
    // then the partial sums of each digit meet in shared memory. With chunk
    // sums, the whole chunks before this tile's chunk are one row each.
    __shared__ uint4 partial[kRowLanes][kSweepBins / 4];
    {
        const uint32_t column = threadIdx.x & 63u;
        const uint32_t lane_row = threadIdx.x >> 6;
        const uint4* rows = reinterpret_cast<const uint4*>(tile_counts);
        uint4 acc = make_uint4(0, 0, 0, 0);
        uint32_t first_row = 0;
        if (chunk_sums != nullptr) {
            const uint4* chunk_rows = reinterpret_cast<const uint4*>(chunk_sums);
            const uint32_t chunks = tile / kChunkTiles;
#pragma unroll 8
            for (uint32_t j = lane_row; j < chunks; j += kRowLanes) {
                uint4 c = __ldg(&chunk_rows[static_cast<size_t>(j) * (kSweepBins / 4) + column]);
                acc.x += c.x;
                acc.y += c.y;
                acc.z += c.z;
                acc.w += c.w;
            }
            first_row = chunks * kChunkTiles;
        }
#pragma unroll 8
        for (uint32_t j = first_row + lane_row; j < tile; j += kRowLanes) {
            uint4 c = __ldg(&rows[static_cast<size_t>(j) * (kSweepBins / 4) + column]);
            acc.x += c.x;
            acc.y += c.y;
            acc.z += c.z;
            acc.w += c.w;
        }
        partial[lane_row][column] = acc;
    }
    // Digit base: exclusive scan of the pass histogram (digit-owning warps).
    const uint32_t h = owns_digit ? __ldg(&hist[d]) : 0u;
    uint32_t inc = h;
    if (owns_digit) {
#pragma unroll
        for (uint32_t o = 1; o < 32; o <<= 1) {
            uint32_t u = __shfl_up_sync(0xFFFFFFFFu, inc, o);
            if (lane >= o) {
                inc += u;
            }
        }
        if (lane == 31) {
            scan_warp[warp] = inc;
        }
    }
    __syncthreads();
    const uint32_t below = lanemask_lt();
    const uint32_t base = tile * kSweepTile + warp * (kSweepItems * 32);
    uint32_t key[kSweepItems];
    uint32_t val[kSweepItems];
    uint32_t rank[kSweepItems];
#pragma unroll
    for (uint32_t r = 0; r < kSweepItems; ++r) {
        uint32_t idx = base + r * 32 + lane;
        bool valid = idx < n;
        key[r] = valid ? keys_in[idx] : 0;
        val[r] = valid ? (vals_in != nullptr ? vals_in[idx] : idx) : 0;
    }
#pragma unroll
    for (uint32_t r = 0; r < kSweepItems; ++r) {
        bool valid = base + r * 32 + lane < n;
        uint32_t digit = valid ? (key[r] >> shift) & (kSweepBins - 1) : 0xFFFFFFFFu;
        uint32_t peers = __match_any_sync(0xFFFFFFFFu, digit);
        uint32_t prior = valid ? warp_counts[warp][digit] : 0;
        rank[r] = valid ? prior + static_cast<uint32_t>(__popc(peers & below)) : 0xFFFFFFFFu;
        __syncwarp();
        if (valid && lane == static_cast<uint32_t>(__ffs(peers) - 1)) {
            warp_counts[warp][digit] = prior + static_cast<uint32_t>(__popc(peers));
        }
        __syncwarp();
    }
    __syncthreads();
    if (owns_digit) {
        uint32_t running = 0;
#pragma unroll
        for (uint32_t w = 0; w < kWarps; ++w) {
            uint32_t c = warp_counts[w][d];
            warp_counts[w][d] = running;
            running += c;
        }
        uint32_t warp_base = 0;
        for (uint32_t w = 0; w < warp; ++w) {
            warp_base += scan_warp[w];
        }
        const uint32_t* flat = reinterpret_cast<const uint32_t*>(&partial[0][0]);
        uint32_t before = 0;
#pragma unroll
        for (uint32_t l = 0; l < kRowLanes; ++l) {
            before += flat[l * kSweepBins + d];
        }
        digit_offset[d] = warp_base + inc - h + before;
    }
    __syncthreads();
#pragma unroll
    for (uint32_t r = 0; r < kSweepItems; ++r) {
        const bool valid = rank[r] != 0xFFFFFFFFu;
        uint32_t slot = 0xFFFFFFFFu;  // next-pass count this key adds to
        if (valid) {
            uint32_t digit = (key[r] >> shift) & (kSweepBins - 1);
            uint32_t dst = digit_offset[digit] + warp_counts[warp][digit] + rank[r];
            keys_out[dst] = key[r];
            vals_out[dst] = val[r];
            slot = (dst / kSweepTile) * kSweepBins + ((key[r] >> next_shift) & (kSweepBins - 1));
        }
        if (next_counts != nullptr) {
            if (kAggregate) {
                const uint32_t peers = __match_any_sync(0xFFFFFFFFu, slot);
                if (valid && lane == static_cast<uint32_t>(__ffs(peers) - 1)) {
                    atomicAdd(&next_counts[slot], static_cast<uint32_t>(__popc(peers)));
                }
            } else if (valid) {
                atomicAdd(&next_counts[slot], 1u);
            }
        }
    }
}

}  // namespace

size_t onesweep_scratch_words(uint32_t n, uint32_t passes) {
    const size_t tiles = sweep_tiles(n == 0 ? 1 : n);
    const size_t words32 = static_cast<size_t>(passes) * tiles * kSweepBins + static_cast<size_t>(passes) * kSweepBins +
                           static_cast<size_t>(sweep_chunks(static_cast<uint32_t>(tiles))) * kSweepBins;
    return (words32 + 1) / 2;
}

namespace {

cudaError_t keys_and_counts(const float4* pos, const uint16_t* tank_of, const TankConst* tanks, uint32_t n,
                            uint32_t* keys, uint32_t passes, unsigned long long* sweep, uint32_t morton_bits,
                            const uint32_t* ids, cudaStream_t stream, bool hilbert = false,
                            IdSplit split = IdSplit{}, uint32_t split_at = 0) {
    cudaError_t err = cudaMemsetAsync(sweep, 0, onesweep_scratch_words(n, passes) * sizeof(unsigned long long), stream);
    if (err != cudaSuccess) {
        return err;
    }
    const uint32_t tiles = sweep_tiles(n);
    SweepLayout l = sweep_layout(sweep, tiles, passes);
    if (morton_bits != 0) {
        keys_hist_kernel<true><<<tiles, kKeysThreads, 0, stream>>>(pos, tank_of, tanks, n, keys, passes, l.tile_counts,
                                                                   l.hist, morton_bits, ids, hilbert ? 1 : 0,
                                                                   split, split_at);
    } else {
        keys_hist_kernel<false><<<tiles, kKeysThreads, 0, stream>>>(pos, tank_of, tanks, n, keys, passes,
                                                                    l.tile_counts, l.hist, 0, ids, 0, IdSplit{}, 0);
    }
    return cudaGetLastError();
}

// ---- a curve order by counting (one tank) ----------------------------------
//
// The processing order needs locality, not a sorted sequence: particles are
// grouped by the curve code of a coarsened cell (2^shift cells a side) with
// one atomic place each, the groups laid out in curve order by a scan of
// their counts, and a group's particles take its slots in the atomics' order.

__device__ __forceinline__ uint32_t coarse_curve_key(float4 p, const TankConst* t, uint32_t axis_bits, uint32_t shift,
                                                     bool hilbert) {
    const float h = __ldg(&t->h);
    const int limit = static_cast<int>((1u << axis_bits) - 1u);
    const uint32_t cx = static_cast<uint32_t>(min(max(cell_coord(p.x, h) - cell_coord(__ldg(&t->low[0]), h), 0), limit)) >> shift;
    const uint32_t cy = static_cast<uint32_t>(min(max(cell_coord(p.y, h) - cell_coord(__ldg(&t->low[1]), h), 0), limit)) >> shift;
    const uint32_t cz = static_cast<uint32_t>(min(max(cell_coord(p.z, h) - cell_coord(__ldg(&t->low[2]), h), 0), limit)) >> shift;
    const uint32_t bits = axis_bits - shift;
    return hilbert ? hilbert3(cx, cy, cz, bits) : spread3(cx) | (spread3(cy) << 1) | (spread3(cz) << 2);
}

__global__ void __launch_bounds__(256) curve_count_kernel(const float4* __restrict__ pos,
                                                          const TankConst* __restrict__ tanks, uint32_t n,
                                                          uint32_t axis_bits, uint32_t shift, int hilbert,
                                                          uint32_t* __restrict__ keys, uint32_t* __restrict__ within,
                                                          uint32_t* __restrict__ counts) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) {
        return;
    }
    const uint32_t key = coarse_curve_key(pos[i], tanks, axis_bits, shift, hilbert != 0);
    keys[i] = key;
    within[i] = atomicAdd(&counts[key], 1u);
}

// A batch's processing order: each tank's cells in row order (x fastest)
// from curve_base; a particle takes a place in its cell's bin with one atomic.
__global__ void __launch_bounds__(256) tank_cells_count_kernel(const float4* __restrict__ pos,
                                                               const uint16_t* __restrict__ tank_of,
                                                               const TankConst* __restrict__ tanks, uint32_t n,
                                                               uint32_t* __restrict__ keys,
                                                               uint32_t* __restrict__ within,
                                                               uint32_t* __restrict__ counts) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) {
        return;
    }
    const TankConst* t = tanks + tank_of[i];
    const float4 p = pos[i];
    const float h = __ldg(&t->h);
    const int nx = static_cast<int>(__ldg(&t->curve_dims[0]));
    const int ny = static_cast<int>(__ldg(&t->curve_dims[1]));
    const int nz = static_cast<int>(__ldg(&t->curve_dims[2]));
    const int cx = min(max(cell_coord(p.x, h) - cell_coord(__ldg(&t->low[0]), h), 0), nx - 1);
    const int cy = min(max(cell_coord(p.y, h) - cell_coord(__ldg(&t->low[1]), h), 0), ny - 1);
    const int cz = min(max(cell_coord(p.z, h) - cell_coord(__ldg(&t->low[2]), h), 0), nz - 1);
    const uint32_t key = __ldg(&t->curve_base) + static_cast<uint32_t>((cz * ny + cy) * nx + cx);
    keys[i] = key;
    within[i] = atomicAdd(&counts[key], 1u);
}

__global__ void __launch_bounds__(256) curve_rank_kernel(const uint32_t* __restrict__ keys,
                                                         const uint32_t* __restrict__ within, uint32_t n,
                                                         const uint2* __restrict__ ranges, uint32_t* __restrict__ rank) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        rank[i] = __ldg(&ranges[keys[i]]).x + within[i];
    }
}

}  // namespace

cudaError_t launch_keys_onesweep(const float4* pos, const uint16_t* tank_of, const TankConst* tanks, uint32_t n,
                                 uint32_t* keys, uint32_t passes, unsigned long long* sweep, cudaStream_t stream,
                                 const uint32_t* ids) {
    if (n == 0) {
        return cudaSuccess;
    }
    return keys_and_counts(pos, tank_of, tanks, n, keys, passes, sweep, 0, ids, stream);
}

cudaError_t launch_morton_rank(const float4* pos, const uint16_t* tank_of, const TankConst* tanks, uint32_t n,
                               uint32_t morton_bits, uint32_t key_bits, GridScratch scratch,
                               unsigned long long* sweep, uint32_t* rank, cudaStream_t stream, uint32_t* launches,
                               bool hilbert, const uint32_t* ids, const IdSplit& split) {
    if (n == 0) {
        return cudaSuccess;
    }
    const uint32_t split_bits = split.count > 1 ? bit_width32(split.count - 1u) : 0u;
    bool ranges_ok = split.count <= IdSplit::kMax && (split.count <= 1 || (split.start[0] == 0 && split.start[split.count] == n));
    for (uint32_t c = 0; ranges_ok && split.count > 1 && c < split.count; ++c) {
        ranges_ok = split.start[c] < split.start[c + 1];
    }
    if (morton_bits == 0 || morton_bits > 10 || key_bits + split_bits > 32 || !ranges_ok) {
        return cudaErrorInvalidValue;
    }
    const uint32_t split_at = key_bits;
    key_bits += split_bits;
    const uint32_t passes = onesweep_passes(key_bits);
    if (passes > kSweepMaxPasses) {
        return cudaErrorInvalidValue;
    }
    cudaError_t err =
        keys_and_counts(pos, tank_of, tanks, n, scratch.keys, passes, sweep, morton_bits, ids, stream, hilbert,
                        split, split_at);
    if (err == cudaSuccess) {
        err = launch_onesweep_sort(scratch, n, passes, sweep, stream, launches, true);
    }
    if (err != cudaSuccess) {
        return err;
    }
    rank_kernel<<<(n + 255) / 256, 256, 0, stream>>>(scratch.sorted_ids, n, rank, ids);
    if (launches != nullptr) {
        *launches += 2;
    }
    return cudaGetLastError();
}

namespace {

// ids[compact_base + j] = global_base + j for each range (one block per range).
__global__ void __launch_bounds__(256) compact_ids_kernel(const uint32_t* __restrict__ ranges, uint32_t* __restrict__ ids) {
    const uint32_t global_base = ranges[3 * blockIdx.x];
    const uint32_t compact_base = ranges[3 * blockIdx.x + 1];
    const uint32_t count = ranges[3 * blockIdx.x + 2];
    for (uint32_t j = threadIdx.x; j < count; j += blockDim.x) {
        ids[compact_base + j] = global_base + j;
    }
}

}  // namespace

namespace {

// A chunk of active flags travels as the launch's argument: nothing to copy
// (and nothing for the host to wait on) before the launch.
constexpr uint32_t kFlagChunk = 2048;
struct FlagChunk {
    uint32_t first;
    uint32_t count;
    uint8_t flag[kFlagChunk];
};

__global__ void __launch_bounds__(256) set_active_kernel(TankConst* __restrict__ tanks, const FlagChunk chunk) {
    for (uint32_t j = threadIdx.x; j < chunk.count; j += blockDim.x) {
        tanks[chunk.first + j].active = chunk.flag[j] != 0 ? 1u : 0u;
    }
}

}  // namespace

cudaError_t launch_set_active(TankConst* tanks, const uint8_t* active, uint32_t count, cudaStream_t stream) {
    for (uint32_t first = 0; first < count; first += kFlagChunk) {
        FlagChunk chunk;
        chunk.first = first;
        chunk.count = count - first < kFlagChunk ? count - first : kFlagChunk;
        std::memcpy(chunk.flag, active + first, chunk.count);
        set_active_kernel<<<1, 256, 0, stream>>>(tanks, chunk);
        cudaError_t err = cudaGetLastError();
        if (err != cudaSuccess) {
            return err;
        }
    }
    return cudaSuccess;
}

cudaError_t launch_compact_ids(const uint32_t* ranges, uint32_t range_count, uint32_t* ids, cudaStream_t stream) {
    if (range_count == 0) {
        return cudaSuccess;
    }
    compact_ids_kernel<<<range_count, 256, 0, stream>>>(ranges, ids);
    return cudaGetLastError();
}

cudaError_t launch_onesweep_sort(GridScratch& s, uint32_t n, uint32_t passes, unsigned long long* sweep,
                                 cudaStream_t stream, uint32_t* launches, bool aggregate) {
    if (n == 0) {
        s.sorted_keys = s.keys_a;
        s.sorted_ids = s.vals_a;
        return cudaSuccess;
    }
    const uint32_t tiles = sweep_tiles(n);
    SweepLayout l = sweep_layout(sweep, tiles, passes);
    const uint32_t* kin = s.keys;
    const uint32_t* vin = nullptr;
    uint32_t* kout = s.keys_a;
    uint32_t* vout = s.vals_a;
    const bool chunked = tiles > kChunkedTiles;
    for (uint32_t p = 0; p < passes; ++p) {
        uint32_t* next = p + 1 < passes ? l.tile_counts + static_cast<size_t>(p + 1) * tiles * kSweepBins : nullptr;
        const uint32_t* counts = l.tile_counts + static_cast<size_t>(p) * tiles * kSweepBins;
        const uint32_t* hist = l.hist + static_cast<size_t>(p) * kSweepBins;
        if (chunked) {
            chunk_sums_kernel<<<sweep_chunks(tiles), kSweepBins, 0, stream>>>(counts, tiles, l.chunk_sums);
            if (launches != nullptr) {
                *launches += 1;
            }
        }
        const uint32_t* chunk_sums = chunked ? l.chunk_sums : nullptr;
        if (aggregate) {
            sweep_scatter_kernel<true><<<tiles, kSweepThreads, 0, stream>>>(kin, vin, kout, vout, n, p * kSweepBits,
                                                                            hist, counts, next, (p + 1) * kSweepBits,
                                                                            chunk_sums);
        } else {
            sweep_scatter_kernel<false><<<tiles, kSweepThreads, 0, stream>>>(kin, vin, kout, vout, n, p * kSweepBits,
                                                                             hist, counts, next, (p + 1) * kSweepBits,
                                                                             chunk_sums);
        }
        if (launches != nullptr) {
            *launches += 1;
        }
        kin = kout;
        vin = vout;
        if (kout == s.keys_a) {
            kout = s.keys_b;
            vout = s.vals_b;
        } else {
            kout = s.keys_a;
            vout = s.vals_a;
        }
    }
    s.sorted_keys = kin;
    s.sorted_ids = vin;
    return cudaGetLastError();
}

RadixPlan plan_radix(uint32_t key_bits, uint32_t digit_bits) {
    RadixPlan plan;
    digit_bits = digit_bits < 1 ? 1 : (digit_bits > kRadixMaxBits ? kRadixMaxBits : digit_bits);
    if (key_bits == 0) {
        key_bits = 1;
    }
    uint32_t passes = (key_bits + digit_bits - 1) / digit_bits;
    if (passes > 8) {
        passes = 8;
    }
    // Spread the bits evenly so no pass carries a nearly empty digit.
    uint32_t shift = 0;
    for (uint32_t p = 0; p < passes; ++p) {
        uint32_t remaining = key_bits - shift;
        uint32_t width = (remaining + (passes - p) - 1) / (passes - p);
        plan.shift[p] = shift;
        plan.bits[p] = width;
        shift += width;
    }
    plan.passes = passes;
    return plan;
}

size_t counting_block_sums(uint32_t buckets) { return (static_cast<size_t>(buckets) + kScanTile - 1) / kScanTile; }

cudaError_t launch_counting_grid(const float4* pos, const uint16_t* tank_of, const TankConst* tanks, uint32_t n,
                                 uint32_t buckets, GridScratch& s, uint32_t* counts, uint32_t* block_sums,
                                 uint2* bucket, cudaStream_t stream, uint32_t* launches) {
    s.sorted_keys = nullptr;
    s.sorted_ids = s.vals_b;
    cudaError_t e = cudaMemsetAsync(counts, 0, sizeof(uint32_t) * buckets, stream);
    if (e != cudaSuccess) {
        return e;
    }
    const uint32_t particle_blocks = (n + 255) / 256;
    const uint32_t scan_blocks = static_cast<uint32_t>(counting_block_sums(buckets));
    if (n > 0) {
        count_keys_kernel<<<particle_blocks, 256, 0, stream>>>(pos, tank_of, tanks, n, s.keys, s.keys_a, counts);
    }
    scan_reduce_kernel<<<scan_blocks, 256, 0, stream>>>(counts, buckets, block_sums);
    scan_top_kernel<<<1, 1024, 0, stream>>>(block_sums, scan_blocks);
    scan_down_kernel<<<scan_blocks, 256, 0, stream>>>(counts, buckets, block_sums, bucket);
    if (n > 0) {
        place_kernel<<<particle_blocks, 256, 0, stream>>>(s.keys, s.keys_a, n, bucket, s.vals_a);
    }
    if (launches != nullptr) {
        *launches += n > 0 ? 5 : 3;
    }
    return cudaGetLastError();
}

cudaError_t launch_curve_rank_counting(const float4* pos, const TankConst* tanks, uint32_t n, uint32_t axis_bits,
                                      uint32_t shift, bool hilbert, uint32_t* keys, uint32_t* within,
                                      uint32_t* counts, uint32_t* block_sums, uint2* ranges, uint32_t* rank,
                                      cudaStream_t stream, uint32_t* launches) {
    if (n == 0) {
        return cudaSuccess;
    }
    if (axis_bits == 0 || axis_bits > 10 || shift >= axis_bits) {
        return cudaErrorInvalidValue;
    }
    const uint32_t bins = 1u << (3u * (axis_bits - shift));
    cudaError_t e = cudaMemsetAsync(counts, 0, sizeof(uint32_t) * bins, stream);
    if (e != cudaSuccess) {
        return e;
    }
    const uint32_t blocks = (n + 255) / 256;
    const uint32_t scan_blocks = static_cast<uint32_t>(counting_block_sums(bins));
    curve_count_kernel<<<blocks, 256, 0, stream>>>(pos, tanks, n, axis_bits, shift, hilbert ? 1 : 0, keys, within,
                                                   counts);
    scan_reduce_kernel<<<scan_blocks, 256, 0, stream>>>(counts, bins, block_sums);
    scan_top_kernel<<<1, 1024, 0, stream>>>(block_sums, scan_blocks);
    scan_down_kernel<<<scan_blocks, 256, 0, stream>>>(counts, bins, block_sums, ranges);
    curve_rank_kernel<<<blocks, 256, 0, stream>>>(keys, within, n, ranges, rank);
    if (launches != nullptr) {
        *launches += 5;
    }
    return cudaGetLastError();
}

cudaError_t launch_tank_cells_rank(const float4* pos, const uint16_t* tank_of, const TankConst* tanks, uint32_t n,
                                   uint32_t bins, uint32_t* keys, uint32_t* within, uint32_t* counts,
                                   uint32_t* block_sums, uint2* ranges, uint32_t* rank, cudaStream_t stream,
                                   uint32_t* launches) {
    if (n == 0) {
        return cudaSuccess;
    }
    if (bins == 0 || tank_of == nullptr) {
        return cudaErrorInvalidValue;
    }
    cudaError_t e = cudaMemsetAsync(counts, 0, sizeof(uint32_t) * bins, stream);
    if (e != cudaSuccess) {
        return e;
    }
    const uint32_t blocks = (n + 255) / 256;
    const uint32_t scan_blocks = static_cast<uint32_t>(counting_block_sums(bins));
    tank_cells_count_kernel<<<blocks, 256, 0, stream>>>(pos, tank_of, tanks, n, keys, within, counts);
    scan_reduce_kernel<<<scan_blocks, 256, 0, stream>>>(counts, bins, block_sums);
    scan_top_kernel<<<1, 1024, 0, stream>>>(block_sums, scan_blocks);
    scan_down_kernel<<<scan_blocks, 256, 0, stream>>>(counts, bins, block_sums, ranges);
    curve_rank_kernel<<<blocks, 256, 0, stream>>>(keys, within, n, ranges, rank);
    if (launches != nullptr) {
        *launches += 5;
    }
    return cudaGetLastError();
}

cudaError_t launch_gather_vel(const uint32_t* sorted_ids, uint32_t n, const float4* vel, float4* svel,
                              cudaStream_t stream) {
    if (n == 0) {
        return cudaSuccess;
    }
    gather_vel_kernel<<<(n + 255) / 256, 256, 0, stream>>>(sorted_ids, n, vel, svel);
    return cudaGetLastError();
}

cudaError_t launch_order_gather(const GridScratch& s, uint32_t n, const uint2* bucket, uint32_t* counts,
                                const float4* pos, const float4* vel, const uint16_t* tank_of, float4* spos,
                                float4* svel, uint16_t* stank, const Schedule& schedule, cudaStream_t stream) {
    if (n == 0) {
        return cudaSuccess;
    }
    order_gather_kernel<<<(n + 255) / 256, 256, 0, stream>>>(s.keys, s.vals_a, n, bucket, counts, s.vals_b, pos, vel,
                                                             tank_of, spos, svel, stank, schedule);
    return cudaGetLastError();
}

cudaError_t launch_keys(const float4* pos, const uint16_t* tank_of, const TankConst* tanks, uint32_t n, uint32_t* keys,
                        cudaStream_t stream) {
    if (n == 0) {
        return cudaSuccess;
    }
    keys_kernel<<<(n + 255) / 256, 256, 0, stream>>>(pos, tank_of, tanks, n, keys);
    return cudaGetLastError();
}

cudaError_t launch_radix_sort(GridScratch& s, uint32_t n, const RadixPlan& plan, cudaStream_t stream,
                              uint32_t* launches) {
    if (n == 0) {
        s.sorted_keys = s.keys_a;
        s.sorted_ids = s.vals_a;
        return cudaSuccess;
    }
    uint32_t tiles = radix_tiles(n);
    const uint32_t* kin = s.keys;
    const uint32_t* vin = nullptr;
    uint32_t* kout = s.keys_a;
    uint32_t* vout = s.vals_a;
    for (uint32_t p = 0; p < plan.passes; ++p) {
        uint32_t mask = (1u << plan.bits[p]) - 1u;
        radix_upsweep<<<tiles, kRadixThreads, 0, stream>>>(kin, n, plan.shift[p], mask, tiles, s.hist);
        scan_exclusive_block<<<1, 1024, 0, stream>>>(s.hist, (mask + 1) * tiles);
        radix_downsweep<<<tiles, kRadixThreads, 0, stream>>>(kin, vin, kout, vout, n, plan.shift[p], mask, tiles,
                                                             s.hist);
        if (launches != nullptr) {
            *launches += 3;
        }
        kin = kout;
        vin = vout;
        if (kout == s.keys_a) {
            kout = s.keys_b;
            vout = s.vals_b;
        } else {
            kout = s.keys_a;
            vout = s.vals_a;
        }
    }
    s.sorted_keys = kin;
    s.sorted_ids = vin;
    return cudaGetLastError();
}

cudaError_t launch_bounds_gather(const uint32_t* sorted_keys, const uint32_t* sorted_ids, uint32_t n, uint2* bucket,
                                 const float4* pos, const float4* vel, const uint16_t* tank_of, float4* spos,
                                 float4* svel, uint16_t* stank, const Schedule& schedule, cudaStream_t stream,
                                 const uint32_t* ids, uint32_t* global_sorted) {
    if (n == 0) {
        return cudaSuccess;
    }
    bounds_gather_kernel<<<(n + 255) / 256, 256, 0, stream>>>(sorted_keys, sorted_ids, n,
                                                              reinterpret_cast<uint32_t*>(bucket), pos, vel, tank_of,
                                                              spos, svel, stank, schedule, ids, global_sorted);
    return cudaGetLastError();
}

}  // namespace sph
