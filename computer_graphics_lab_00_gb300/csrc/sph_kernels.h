// sph_kernels.h — launchers of the SPH step's CUDA kernels (sm_103a).
//
// Pipeline of one substep (src/physics/fluid_sph.cpp:190-309), all on one
// stream, state in HBM:
//   keys        pos (id order)           -> key[i] = bucket of particle i
//   radix sort  (key, id) stable LSD     -> ids in (bucket, id) order
//   bounds      sorted keys              -> bucket table (start, end)
//   gather      pos, vel by sorted id    -> cell-ordered copies
//   density     27-bucket poly6 sum      -> rho, pressure (cell order)
//   integrate   27-bucket forces + walls -> pos, vel (id order, in place)
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "sph_device.cuh"

namespace sph {

constexpr uint32_t kRadixThreads = 256;
constexpr uint32_t kRadixItems = 16;
constexpr uint32_t kRadixTile = kRadixThreads * kRadixItems;  // 4096 keys per tile
constexpr uint32_t kRadixMaxBits = 8;
constexpr uint32_t kRadixMaxBins = 1u << kRadixMaxBits;

inline uint32_t radix_tiles(uint32_t n) { return (n + kRadixTile - 1) / kRadixTile; }

// One pass plan of the LSD radix sort over keys of `key_bits` bits.
struct RadixPlan {
    uint32_t passes = 0;
    uint32_t shift[8] = {};
    uint32_t bits[8] = {};
};
RadixPlan plan_radix(uint32_t key_bits, uint32_t digit_bits);

// Scratch of the grid build. Sizes: n for the key/id arrays, tiles *
// kRadixMaxBins for the histogram.
struct GridScratch {
    uint32_t* keys = nullptr;    // id order: bucket of particle i
    uint32_t* keys_a = nullptr;  // radix ping-pong
    uint32_t* vals_a = nullptr;
    uint32_t* keys_b = nullptr;
    uint32_t* vals_b = nullptr;
    uint32_t* hist = nullptr;
    // Results of the last sort (point into a or b).
    const uint32_t* sorted_keys = nullptr;
    const uint32_t* sorted_ids = nullptr;
};

// The grid without a radix sort (sort mode 2): one atomic place per particle
// in its bucket and an exclusive scan of the bucket counts (the bucket
// table); launch_order_gather then puts each bucket's 32 smallest ids at its
// front in ascending order and gathers the state there. keys -> s.keys (id
// order), sorted ids -> s.vals_b (s.keys_a, s.vals_a: atomic ranks and the
// unordered placement); s.sorted_keys becomes null. counts: `buckets` words;
// block_sums: counting_block_sums(buckets) words.
size_t counting_block_sums(uint32_t buckets);
cudaError_t launch_counting_grid(const float4* pos, const uint16_t* tank_of, const TankConst* tanks, uint32_t n,
                                 uint32_t buckets, GridScratch& s, uint32_t* counts, uint32_t* block_sums,
                                 uint2* bucket, cudaStream_t stream, uint32_t* launches);

cudaError_t launch_keys(const float4* pos, const uint16_t* tank_of, const TankConst* tanks, uint32_t n, uint32_t* keys,
                        cudaStream_t stream);

// Stable LSD radix sort of (keys, implicit ids 0..n-1). Sets
// scratch.sorted_keys / sorted_ids. `launches` counts kernels enqueued.
cudaError_t launch_radix_sort(GridScratch& scratch, uint32_t n, const RadixPlan& plan, cudaStream_t stream,
                              uint32_t* launches);

// One kernel per 8-bit digit pass. Every pass knows each tile's digit counts
// before it runs (the key kernel counts the first pass's tiles, each pass
// counts the next pass's while it scatters), so a block finds its offsets by
// adding up the counts of the earlier tiles: no block waits on another.
// Scratch: onesweep_scratch_words(n, passes) 64-bit words at `sweep`, zeroed
// by launch_keys_onesweep before every sort.
constexpr uint32_t kSweepBits = 8;
constexpr uint32_t kSweepBins = 1u << kSweepBits;
constexpr uint32_t kSweepMaxPasses = 4;
constexpr uint32_t kSweepThreads = 512;                      // threads of a pass block (the first 256 own a digit each)
constexpr uint32_t kSweepItems = 8;                          // keys per thread in a tile
constexpr uint32_t kSweepTile = kSweepThreads * kSweepItems;  // 4096 keys per tile
inline uint32_t sweep_tiles(uint32_t n) { return (n + kSweepTile - 1) / kSweepTile; }
// Bits to write values up to v (0 for v = 0).
inline uint32_t bit_width32(uint32_t v) {
    uint32_t b = 0;
    while (v != 0) {
        ++b;
        v >>= 1;
    }
    return b;
}

// The particle ids cut into consecutive ranges: range c holds the ids
// [start[c], start[c + 1]), start[0] = 0 and start[count] = n. A processing
// order made with it puts range c's ids in the slots [start[c], start[c + 1])
// (each range in curve order), so a pass over those slots touches only those
// ids' outputs. count 0 or 1: no split.
struct IdSplit {
    static constexpr uint32_t kMax = 8;
    uint32_t count = 0;
    uint32_t start[kMax + 1] = {};
};

inline uint32_t onesweep_passes(uint32_t key_bits) { return key_bits == 0 ? 1 : (key_bits + kSweepBits - 1) / kSweepBits; }
size_t onesweep_scratch_words(uint32_t n, uint32_t passes);
// Keys (as launch_keys) plus the first pass's tile counts and every pass's
// digit histogram; zeroes the scratch first.
// ids (optional): the particles keyed are pos[ids[v]] for v < n (a compacted set).
cudaError_t launch_keys_onesweep(const float4* pos, const uint16_t* tank_of, const TankConst* tanks, uint32_t n,
                                 uint32_t* keys, uint32_t passes, unsigned long long* sweep, cudaStream_t stream,
                                 const uint32_t* ids = nullptr);
// tanks[t].active = active[t] != 0 for every tank (`active` in host memory,
// passed by launch argument).
cudaError_t launch_set_active(TankConst* tanks, const uint8_t* active, uint32_t count, cudaStream_t stream);
// Fills ids from (global_base, compact_base, count) triples, one per range.
cudaError_t launch_compact_ids(const uint32_t* ranges, uint32_t range_count, uint32_t* ids, cudaStream_t stream);
// The digit passes over keys made by launch_keys_onesweep. aggregate: one
// atomic per group of lanes adding to the same count (keys whose digits bunch
// up, as Morton codes of a compact body do).
cudaError_t launch_onesweep_sort(GridScratch& scratch, uint32_t n, uint32_t passes, unsigned long long* sweep,
                                 cudaStream_t stream, uint32_t* launches, bool aggregate = false);

// Processing order of the neighbour passes. When rank is null the passes run
// in sorted (bucket) order. Otherwise rank is a permutation over particle ids
// (the slot of each id in a Morton order of the cells, made by
// launch_morton_rank every few substeps) and bounds_gather writes, for the
// particle at sorted position p with id i, order[rank[i]] = p. The results do
// not depend on the order: every particle's sums run over the same pairs in
// the same sequence whichever thread computes them.
struct Schedule {
    const uint32_t* rank = nullptr;  // n: processing slot of each particle id
    uint32_t* order = nullptr;       // n: sorted positions in processing order
};

// The counting placement's final step (after launch_counting_grid): each
// bucket's 32 smallest ids in ascending order at its front, and the gather
// (vel = null: the velocities are left to launch_gather_vel).
cudaError_t launch_order_gather(const GridScratch& s, uint32_t n, const uint2* bucket, uint32_t* counts,
                                const float4* pos, const float4* vel, const uint16_t* tank_of, float4* spos,
                                float4* svel, uint16_t* stank, const Schedule& schedule, cudaStream_t stream);

// Morton keys of the particles' cells (morton_bits bits per axis, counted
// from each tank's low corner and clamped, the tank index above them), sorted
// with the one-kernel passes in the sort buffers of `scratch` (a copy: the
// caller's grid pointers stay as they were), then rank[id] = slot.
// hilbert: the cells' Hilbert index (Skilling's transpose form) instead of
// their Morton code. ids (optional): order the compacted set pos[ids[v]],
// v < n; rank is still indexed by particle id (rank[ids[v]] = slot).
// split (count > 1): the particle's id range goes above the curve key, so the
// ids of range c take the slots [split.start[c], split.start[c + 1]).
cudaError_t launch_morton_rank(const float4* pos, const uint16_t* tank_of, const TankConst* tanks, uint32_t n,
                               uint32_t morton_bits, uint32_t key_bits, GridScratch scratch,
                               unsigned long long* sweep, uint32_t* rank, cudaStream_t stream, uint32_t* launches,
                               bool hilbert = false, const uint32_t* ids = nullptr, const IdSplit& split = IdSplit{});

// Processing order of one tank by counting: particles grouped by the curve
// code (Morton, or Hilbert when `hilbert`) of their cell coarsened by 2^shift
// a side (axis_bits - shift bits an axis), the groups in curve order, a
// group's particles in the order of their atomic places; rank[id] = slot.
// Scratch: keys and within (n words each), counts (zero or not; the bins are
// zeroed first and left zero), block_sums (counting_block_sums(bins)),
// ranges (bins = 2^(3 (axis_bits - shift)) entries).
cudaError_t launch_curve_rank_counting(const float4* pos, const TankConst* tanks, uint32_t n, uint32_t axis_bits,
                                      uint32_t shift, bool hilbert, uint32_t* keys, uint32_t* within,
                                      uint32_t* counts, uint32_t* block_sums, uint2* ranges, uint32_t* rank,
                                      cudaStream_t stream, uint32_t* launches);

// Processing order of a batch by counting: each tank's cells in row order (x
// fastest, TankConst::curve_dims cells a side) from TankConst::curve_base, a
// cell's particles in the order of their atomic places; rank[id] = slot.
// bins: the tanks' cells in all. Scratch as launch_curve_rank_counting.
cudaError_t launch_tank_cells_rank(const float4* pos, const uint16_t* tank_of, const TankConst* tanks, uint32_t n,
                                   uint32_t bins, uint32_t* keys, uint32_t* within, uint32_t* counts,
                                   uint32_t* block_sums, uint2* ranges, uint32_t* rank, cudaStream_t stream,
                                   uint32_t* launches);

// svel[p].xyz = vel[sorted_ids[p]].xyz, .w untouched: the velocities of a
// gather launched with vel = null (the density pass may run meanwhile).
cudaError_t launch_gather_vel(const uint32_t* sorted_ids, uint32_t n, const float4* vel, float4* svel,
                              cudaStream_t stream);

// Bucket table (start, end) from sorted keys (table pre-zeroed), the
// cell-ordered copies of position, velocity and tank id, and (with a
// schedule) the processing order.
// With `ids` the sorted entries index a compacted set: the particle is
// ids[entry], and global_sorted[p] receives its id for the write-back.
// vel = null leaves the sorted velocities to launch_gather_vel.
cudaError_t launch_bounds_gather(const uint32_t* sorted_keys, const uint32_t* sorted_ids, uint32_t n, uint2* bucket,
                                 const float4* pos, const float4* vel, const uint16_t* tank_of, float4* spos,
                                 float4* svel, uint16_t* stank, const Schedule& schedule, cudaStream_t stream,
                                 const uint32_t* ids = nullptr, uint32_t* global_sorted = nullptr);

// Shape of the neighbour passes. variant 0: one thread per particle with
// nested bucket loops; 1: flat candidate stream (density) and the queued pair
// pass (integrate); 2: density records each particle's in-range pairs and
// integrate runs only those; 3: as 2 with divisions through a shared
// correctly rounded reciprocal; 4: density stores per-bucket 32-bit masks
// of the pairs integrate uses (bucket-major, coalesced) and integrate expands
// them (reciprocal divisions); 5: cell-cooperative (a warp's particles of one
// cell share a candidate list in shared memory; density stores chunk-major
// masks over that list, 27 words per particle at most, and integrate
// computes the listed pairs one per lane); 6: the masks of 4, and an
// integrate that stages every bucket its block visits in shared memory once
// (block 128 or 256). block: threads per block of integrate
// (64/128/256 for variants 2-3); queue: in-range pairs buffered per thread
// (variant 1: 8, 16, 24 or 32). pair_list / pair_count / list_cap: the
// per-particle pair lists of variants 2-3 (device buffers the engine owns).
struct NeighbourTuning {
    uint32_t variant = 4;
    uint32_t block = 128;
    uint32_t queue = 32;
    uint16_t* pair_list = nullptr;
    uint16_t* pair_count = nullptr;
    uint32_t list_cap = 64;
    uint32_t* masks = nullptr;  // 27 words per particle, bucket-major (variant 4)
    const uint32_t* order = nullptr;  // processing order (null: sorted order)
    bool all_tanks = false;           // density of inactive tanks too (variant 4 skips them otherwise)
    // Integrate only the processing slots [slot_begin, min(slot_end, n))
    // (variant 4; the other variants take the whole range only).
    uint32_t slot_begin = 0;
    uint32_t slot_end = 0xFFFFFFFFu;
    // Variant 4's integrate launched as a programmatic dependent of the
    // launch before it in the stream (which must write nothing it reads).
    bool programmatic = false;
};

// Density and pressure (fluid_sph.cpp:200-222). Writes spos2 = (xyz, rho)
// and svel[p].w = pressure. `counters` may be null (no pair counting).
cudaError_t launch_density(const float4* spos, float4* svel, float4* spos2, const uint2* bucket, const TankConst* tanks,
                           const uint16_t* stank, uint32_t n, StepCounters* counters, cudaStream_t stream,
                           const NeighbourTuning& tuning);

// Forces, semi-implicit Euler, speed clamp and walls (fluid_sph.cpp:225-305).
// Writes the id-order state.
// dst[ids[p]] = src[p] for p < n (sorted order to id order).
cudaError_t launch_scatter_rows(const float4* src, const uint32_t* ids, uint32_t n, float4* dst, cudaStream_t stream);

// Sets the shared-memory attributes of the staged integrate (variant 6) on the
// current device, once; call before capturing a launch of it.
cudaError_t prepare_staged_integrate();

cudaError_t launch_integrate(const float4* spos2, const float4* svel, const uint32_t* sorted_ids, const uint2* bucket,
                             const TankConst* tanks, const uint16_t* stank, uint32_t n, float4* pos, float4* vel,
                             cudaStream_t stream, const NeighbourTuning& tuning);

// FluidSolver::emit lattice (fluid_sph.cpp:138-154) for particles
// [first, first + count) of one tank.
// Force-field accelerations at the substep's start (id order) for tanks with
// fields; shape colliders on the integrated state for tanks with colliders.
cudaError_t launch_fields(const float4* pos, const uint16_t* tank_of, const TankConst* tanks, uint32_t n,
                          float4* out, cudaStream_t stream);
cudaError_t launch_colliders(float4* pos, float4* vel, const uint16_t* tank_of, const TankConst* tanks, uint32_t n,
                             cudaStream_t stream);
cudaError_t launch_emit(const TankConst* tank, uint32_t first, uint32_t count, float4* pos, float4* vel, float4* prev,
                        cudaStream_t stream);

// FP64 per-tank statistics of the id-order state. acc holds 10 doubles per
// tank: sum rho, sum compression, max rho (as bits), com xyz, kinetic,
// nonfinite count, count.
constexpr uint32_t kStatsPerTank = 10;
cudaError_t launch_stats(const float4* pos, const float4* vel, const uint16_t* tank_of, const TankConst* tanks,
                         uint32_t n, double* acc, cudaStream_t stream);
// Counts particles whose position or velocity xyz is not finite (adds to *out).
cudaError_t launch_count_nonfinite(const float4* pos, const float4* vel, uint32_t n, uint32_t* out, cudaStream_t stream);
// Learned coarse step, first half: the plain SPH force per particle
// (force[p], sorted order) and the 32 correction features (row p, or row
// sorted_ids[p] when id_order). Needs the variant-4 pair masks of density.
// With x_tiles the features go instead to the MLP's input tiles, normalised
// by (norm_mean, norm_inv_std) and rounded to BF16 (row p); with neither
// features nor x_tiles only the force is written.
cudaError_t launch_features(const float4* spos2, const float4* svel, const uint32_t* sorted_ids, const uint2* bucket,
                            const TankConst* tanks, const uint16_t* stank, uint32_t n, const uint32_t* order,
                            const uint32_t* masks, float4* force, float* features, bool id_order,
                            cudaStream_t stream, const float* norm_mean = nullptr,
                            const float* norm_inv_std = nullptr, uint8_t* x_tiles = nullptr);
// Net correction of each active tank: kCorrectionSumWords unsigned words per
// tank (x, y, z sums in 2^-24 fixed point, two's complement, and the count),
// zeroed first. Deterministic: integer sums do not depend on atomic order.
// programmatic: launched as a programmatic dependent of the MLP, the sums
// already zeroed (zero_correction_sums, earlier in the stream).
constexpr uint32_t kCorrectionSumWords = 4;
cudaError_t zero_correction_sums(uint32_t tank_count, unsigned long long* sums, cudaStream_t stream);
cudaError_t launch_correction_sums(const float4* correction, const TankConst* tanks, const uint16_t* stank, uint32_t n,
                                   uint32_t tank_count, unsigned long long* sums, cudaStream_t stream,
                                   bool programmatic = false);
// Second half: acceleration = plain + correction[p] (null: none), minus the
// tank's mean correction along the axes in `free_axes` (bit a: axis a) when
// `sums` (launch_correction_sums) is given, then the plain step's velocity
// update, clamp, walls and id-order write. programmatic: launched as a
// programmatic dependent of the kernel before it (features, MLP or sums).
cudaError_t launch_finish_learned(const float4* spos2, const float4* svel, const uint32_t* sorted_ids,
                                  const TankConst* tanks, const uint16_t* stank, uint32_t n, const float4* force,
                                  const float4* correction, const unsigned long long* sums, uint32_t free_axes,
                                  float4* pos, float4* vel, cudaStream_t stream,
                                  bool programmatic = false);
// Counts x / y (over `count` generated pairs) where division through a
// correctly rounded reciprocal differs from IEEE division. mode 0: every
// divisor mantissa; mode 1: random signs, mantissas, exponents.
cudaError_t launch_division_selftest(uint64_t seed, uint64_t count, int mode, unsigned long long* mismatches,
                                     cudaStream_t stream);
// Largest bucket count and number of buckets above capacity.
cudaError_t launch_bucket_stats(const uint2* bucket, uint32_t buckets, uint32_t* out2, cudaStream_t stream);

}  // namespace sph
