// sph_engine.h — host-side owner of the device state of one or more tanks.
//
// A tank is one independent fluid (the reference's FluidSolver,
// src/physics/fluid_sph.h:101-127). The engine keeps all tanks' particles in
// one id-ordered array (tank t owns [particle_base, particle_base + count)),
// and all tanks' bucket tables in one global table (tank t owns
// [bucket_base, bucket_base + cells)). One substep advances every active
// tank with the same kernel launches; a single tank is the case T = 1.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/sph_c.h"
#include "sph_kernels.h"
#include "sph_mlp.cuh"
#include "sph_instances.h"
#include "sph_surface.h"

namespace sph {

// Host restatements of the reference's parameter rules.
uint32_t fluid_substeps(const sph_params& params, float delta_seconds);  // fluid_sph.cpp:128-136
TankConst make_tank_const(const sph_params& params, float dt);           // constants of one tank
float sqrt_at_least(float v);  // smallest x >= 0 with sqrtf(x) >= v
float sqrt_at_most(float v);   // largest x >= 0 with sqrtf(x) <= v
int validate_params(const sph_params& params);

// One launch shape and its measured time per substep.
struct TuneChoice {
    NeighbourTuning tuning{};
    uint32_t radix_bits = 6;
    uint32_t schedule = 0;  // processing order: 0 sorted, 1 Morton, 2 Hilbert
    bool onesweep = true;
    bool counting = false;  // grid sort mode 2 (counting placement), over onesweep
    float ms = 0.0F;
};

class Engine {
public:
    // step_host integrates kHostRanges id ranges in turn (the first
    // kHostFirstNum / kHostFirstDen of the ids, then equal parts of the rest)
    // and downloads each range's rows while the next integrates, from
    // kHostOverlapMin particles up.
    static constexpr uint32_t kHostRanges = 3;
    static constexpr uint32_t kHostFirstNum = 1;
    static constexpr uint32_t kHostFirstDen = 2;
    static constexpr uint32_t kHostOverlapMin = 1u << 18;
    ~Engine();

    // Allocates for `tanks` tanks with the given capacities (particles) and
    // bucket counts. Returns a status code.
    int init(int device, const std::vector<sph_params>& params, const std::vector<uint32_t>& capacities);

    int set_params(uint32_t tank, const sph_params& params);
    int upload(uint32_t tank, const float* pos, const float* vel, uint32_t count);
    int download(uint32_t tank, float* pos, float* vel);
    int download_previous(uint32_t tank, float* pos);
    int keep_rendered();
    // Draw instances of tank 0's particles into caller device buffers, then keep_rendered.
    int write_instances(sph_instance* instances, uint32_t instance_base, uint32_t sphere_mesh,
                        sph_tlas_instance* tlas, uint32_t tlas_base, uint64_t blas, uint32_t fluid_index,
                        uint32_t flags);
    int emit(uint32_t tank, uint32_t count);
    // upload + run + download of a single tank in one call, with the
    // velocity upload overlapping the first substep's keys and sort; same
    // results and checks. pos_out / vel_out may alias the inputs or be null.
    int step_host(const float* pos_in, const float* vel_in, uint32_t count, float dt, uint32_t substeps,
                  float* pos_out, float* vel_out);

    // Enqueues `substeps` substeps of length dt for every active tank.
    int run(float dt, uint32_t substeps);
    // Tank t runs substeps[t] substeps of length dt[t] (tanks that finish
    // early sit out the remaining rounds).
    int run_per_tank(const std::vector<float>& dt, const std::vector<uint32_t>& substeps);
    // FP64 statistics of every tank.
    int stats_all(std::vector<sph_stats>& out);
    // Times candidate launch shapes on the current state (restored after)
    // and keeps the fastest. Results never depend on the shape.
    int autotune(float dt, uint32_t substeps, TuneChoice* best, std::vector<TuneChoice>* tried);
    // Learned coarse substeps: plain force + MLP correction (model may be
    // null: zero correction, bit-identical to the plain substep).
    int run_learned(float dt, uint32_t substeps, const mlp::ModelView* model);
    // Correction features of the current state, id order, n x 32 (device).
    int learned_features(float dt, float* features);
    int learned_correction(float dt, const mlp::ModelView& model, float4* correction);
    // SPH_ERR_TIMEOUT if a tensor-core wait gave up since the last check.
    int learned_error();
    uint32_t learned_launches_per_substep() const { return learned_launches_; }
    // Saves (true) or restores (false) the particle state in device memory,
    // in one of kSnapshotSlots slots; restore_tanks copies back only the
    // particles of the tanks with which[t] != 0.
    static constexpr uint32_t kSnapshotSlots = 2;
    int snapshot(bool save, uint32_t slot = 0);
    int restore_tanks(uint32_t slot, const std::vector<uint8_t>& which);
    // Device-to-device copy of the whole state (id order) into caller buffers.
    int copy_state(float4* positions, float4* velocities);
    // Grid build only (for inspection).
    int build_grid();
    int grid_download(uint32_t tank, uint32_t* cell_of, uint32_t* cell_counts, uint32_t* cell_particles);
    int stats(uint32_t tank, sph_stats* out, bool with_pairs);
    int synchronize();
    int set_active(const std::vector<uint8_t>& active);
    int set_radix_bits(uint32_t bits);
    int set_tuning(const NeighbourTuning& tuning);
    int set_schedule(uint32_t curve);  // 0 sorted order, 1 Morton, 2 Hilbert
    uint32_t schedule_on() const { return schedule_curve_; }
    // Grid sort: one kernel per 8-bit digit pass, or three kernels per
    // radix_bits-wide pass.
    int set_onesweep(bool on);
    bool onesweep_on() const { return onesweep_; }
    // Grid sort mode 2: counting placement instead of the radix passes.
    int set_counting(bool on);
    bool counting_on() const { return counting_; }
    int selftest_division(uint64_t seed, uint64_t count, int mode, uint64_t* mismatches);
    const NeighbourTuning& tuning() const { return tuning_; }
    uint32_t radix_bits() const { return radix_bits_; }
    // Fluid surface of one tank (physics::buildFluidField / marchFluidField):
    // the field rebuilds the grid from the current positions; the march cuts
    // the last field into the engine's vertex buffer.
    int surface_field(uint32_t tank, uint32_t resolution);
    int surface_march(float iso, uint32_t capacity, uint32_t* written);
    int surface_field_download(float* out);
    int surface_vertices_download(sph_surface_vertex* out, uint32_t count);
    const float* surface_field_device() const { return surface_field_; }
    const sph_surface_vertex* surface_vertices_device() const { return surface_vertices_; }
    // Runs substeps without the graph, timing each phase with CUDA events on
    // the context stream: keys, sort, bounds+gather, density, integrate.
    static constexpr uint32_t kProfilePhases = 6;
    int profile(float dt, uint32_t substeps, double* phase_ms);

    uint32_t tank_count() const { return static_cast<uint32_t>(tanks_.size()); }
    uint32_t count(uint32_t tank) const { return tanks_[tank].particle_count; }
    uint32_t capacity(uint32_t tank) const { return capacity_[tank]; }
    uint32_t particle_base(uint32_t tank) const { return tanks_[tank].particle_base; }
    uint32_t total_count() const { return total_count_; }
    const sph_params& params(uint32_t tank) const { return params_[tank]; }
    uint32_t launches_per_substep() const { return launches_per_substep_; }
    // Kernels launched by run() (its graphs) and by the processing-order
    // remakes, counted as they are enqueued.
    uint64_t kernels_launched() const { return kernels_launched_; }
    uint64_t device_bytes() const { return device_bytes_; }
    cudaStream_t stream() const { return stream_; }
    float4* positions() const { return pos_; }
    float4* velocities() const { return vel_; }
    const char* last_error() const { return last_error_.c_str(); }
    // Records a CUDA failure and maps it to a status code.
    int fail(cudaError_t error, const char* what);

private:
    int enqueue_grid(uint32_t* launches);
    int enqueue_bounds(uint32_t* launches);
    int enqueue_learned_substep(const mlp::ModelView* model, uint32_t* launches);
    int ensure_learned_buffers();
    int enqueue_substep(uint32_t* launches);
    // Integrate the id ranges of the processing order one by one, an event
    // after each (step_host).
    int enqueue_integrate_ranges();
    int ensure_host_graph();  // captures step_host's overlapped substep
    void drop_host_graph();
    int refresh_constants(float dt);
    void attach_shapes(uint32_t tank);  // copies tank's colliders and fields to staging, sets pointers
    int update_shape_flags();           // has_fields_ / has_colliders_; graphs recaptured on change
    int enqueue_fields(uint32_t* launches);
    int enqueue_colliders(uint32_t* launches);
    int ensure_graph();
    int prepare_schedule(uint32_t* launches);
    void schedule_bits(uint32_t* axis_bits, uint32_t* key_bits) const;
    int run_compact(uint32_t substeps, uint32_t active_particles);
    static constexpr uint32_t kScheduleRefresh = 8;  // grid builds between Morton order refreshes
    static constexpr uint32_t kCountingRefresh = 3;  // the same, one tank's order made by counting
    void release();
    template <typename T> int alloc(T** ptr, size_t count);

    int device_ = 0;
    cudaStream_t stream_ = nullptr;
    std::vector<sph_params> params_;
    std::vector<TankConst> tanks_;
    std::vector<uint32_t> capacity_;
    uint32_t total_capacity_ = 0;
    uint32_t total_count_ = 0;
    uint32_t total_buckets_ = 0;
    uint32_t radix_bits_ = 6;
    RadixPlan plan_{};
    NeighbourTuning tuning_{};
    uint32_t schedule_curve_ = 1;  // processing order: 0 sorted, 1 Morton, 2 Hilbert
    bool capturing_ = false;               // a graph capture is open on stream_
    uint32_t* rank_ = nullptr;             // Morton slot of each particle id (a permutation)
    uint32_t* order_ = nullptr;            // sorted positions in processing order
    uint32_t rank_count_ = 0xFFFFFFFFu;    // particle count rank_ was made for
    uint32_t since_refresh_ = 0;           // grid builds since rank_ was made
    // One tank's curve order by counting (particles grouped by cell, no
    // radix sort) when its cells fit 2^kCurveCountBits a side.
    static constexpr uint32_t kCurveCountBits = 7;
    bool counting_curve_ = true;
    uint2* curve_ranges_ = nullptr;
    size_t curve_capacity_ = 0;  // entries of curve_ranges_
    uint64_t curve_bins_ = 0;    // a batch's cells in all (the tanks' curve_dims products)
    void curve_layout();         // each tank's curve_dims and curve_base, and curve_bins_
    uint32_t want_ranges_ = 0;             // id ranges the next order should carry (step_host), 0: none
    IdSplit rank_split_{};                 // the id ranges rank_ was made with
    uint32_t* compact_ids_ = nullptr;      // ids of the active tanks' particles (a batch run with most tanks idle)
    uint32_t* compact_sorted_ = nullptr;   // their ids in sorted order, for the write-back
    uint32_t* compact_ranges_ = nullptr;   // (global base, compact base, count) per active tank
    std::vector<uint32_t> compact_ranges_host_;
    bool onesweep_ = true;
    bool counting_ = true;
    uint32_t* counts_ = nullptr;      // per bucket: counting placement
    uint32_t* block_sums_ = nullptr;  // its scan's block sums
    unsigned long long* sweep_ = nullptr;  // per-pass tile digit counts and histograms of the one-kernel passes
    float const_dt_ = -1.0f;
    bool consts_dirty_ = true;   // tank table to upload (constants, counts, active flags)
    bool shapes_dirty_ = true;   // collider and force-field tables to upload
    bool active_dirty_ = false;  // only the tanks' active flags changed
    std::vector<uint8_t> active_host_;

    TankConst* d_tanks_ = nullptr;
    sph_collider* d_colliders_ = nullptr;        // SPH_MAX_COLLIDERS per tank
    sph_force_field* d_fields_ = nullptr;        // SPH_MAX_FORCE_FIELDS per tank
    std::vector<sph_collider> colliders_host_;   // staging copies of the same
    std::vector<sph_force_field> fields_host_;
    float4* field_accel_ = nullptr;              // per particle, allocated once some tank has fields
    bool has_fields_ = false;
    bool has_colliders_ = false;
    float4* pos_ = nullptr;
    float4* vel_ = nullptr;
    float4* prev_ = nullptr;
    uint16_t* tank_of_ = nullptr;  // null when there is one tank
    uint16_t* stank_ = nullptr;
    GridScratch grid_{};
    uint2* bucket_ = nullptr;
    float4* spos_ = nullptr;
    float4* spos2_ = nullptr;
    float4* svel_ = nullptr;
    StepCounters* counters_ = nullptr;
    double* stats_acc_ = nullptr;
    uint32_t* bucket_stats_ = nullptr;
    uint64_t device_bytes_ = 0;

    cudaGraphExec_t graph_ = nullptr;
    uint32_t graph_count_ = 0xFFFFFFFFu;
    uint32_t launches_per_substep_ = 0;
    uint64_t kernels_launched_ = 0;
    bool grid_valid_ = false;
    uint32_t nonfinite_host_ = 0;
    cudaStream_t copy_stream_ = nullptr;  // step_host: velocity upload and checks beside the keys and sort
    // step_host: positions landed; velocities landed and checked; sorted ids
    // ready; velocities gathered; then one per integrated id range.
    cudaEvent_t copy_events_[4 + IdSplit::kMax] = {};
    // step_host: id ranges after the first integrate on range_stream_, so
    // their blocks fill the first range's tail; its fork and join events.
    cudaStream_t range_stream_ = nullptr;
    cudaEvent_t range_events_[2] = {};
    cudaGraphExec_t host_graph_ = nullptr;  // step_host's one-substep overlapped form
    uint32_t host_graph_count_ = 0;
    IdSplit host_graph_split_{};
    cudaEvent_t gather_wait_ = nullptr;   // when set, a direct-launched gather first waits for it
    bool defer_vel_ = false;              // a direct-launched gather leaves the velocities out
    uint32_t* flag_host_ = nullptr;       // page-locked non-finite count read back by step_host
    std::vector<uint8_t> user_active_;
    float4* snap_pos_[kSnapshotSlots] = {nullptr, nullptr};
    float4* snap_vel_[kSnapshotSlots] = {nullptr, nullptr};
    float4* sforce_ = nullptr;
    float4* scorrection_ = nullptr;
    uint32_t* compact_rank_ = nullptr;   // processing order of compacted runs (by particle id)
    uint32_t* compact_order_ = nullptr;
    unsigned long long* correction_sums_ = nullptr;  // kCorrectionSumWords per tank
    float* sfeatures_ = nullptr;
    uint8_t* sx_tiles_ = nullptr;  // the MLP's input tiles (learned steps)
    cudaGraphExec_t learned_graph_ = nullptr;
    uint32_t learned_graph_count_ = 0xFFFFFFFFu;
    bool learned_graph_has_model_ = false;
    mlp::ModelView learned_graph_model_{};
    uint32_t learned_launches_ = 0;
    cudaEvent_t events_[8] = {};  // phase boundaries of one profiled substep
    // Surface buffers (grown on demand, byte sizes alongside).
    int grow(void** buffer, size_t* have, size_t need);
    float* surface_field_ = nullptr;
    size_t surface_field_bytes_ = 0;
    void* surface_runs_ = nullptr;  // surface::FieldRuns
    size_t surface_runs_bytes_ = 0;
    uint32_t surface_resolution_ = 0;
    uint32_t surface_tank_ = 0;
    sph_surface_vertex* surface_vertices_ = nullptr;
    size_t surface_vertices_bytes_ = 0;
    uint32_t surface_written_ = 0;
    uint8_t* surface_codes_ = nullptr;
    size_t surface_codes_bytes_ = 0;
    uint32_t* surface_tiles_ = nullptr;  // tile sums, then offsets (tiles + 1), then the limit
    size_t surface_tiles_bytes_ = 0;
    std::string last_error_;
};

}  // namespace sph
