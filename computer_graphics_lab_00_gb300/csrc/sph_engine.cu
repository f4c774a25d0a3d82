// sph_engine.cu — device state, the substep pipeline and its CUDA graph.
#include "sph_engine.h"

#include "sph_mlp.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace sph {

namespace {
// std::numbers::pi_v<float> (fluid_sph.cpp:20).
constexpr float kPi = 3.14159265358979323846F;

// step_host's id ranges for n particles: the first Engine::kHostFirstNum /
// kHostFirstDen of the ids, then the rest in `ranges` - 1 equal parts, every
// cut on a multiple of 128 slots so that each range's mask rows stay
// aligned. No split when n is too small for distinct cuts.
IdSplit host_split(uint32_t n, uint32_t ranges) {
    IdSplit split;
    if (ranges < 2 || ranges > IdSplit::kMax) {
        return split;
    }
    const uint64_t first = static_cast<uint64_t>(n) * Engine::kHostFirstNum / Engine::kHostFirstDen;
    split.count = ranges;
    split.start[0] = 0;
    for (uint32_t c = 1; c < ranges; ++c) {
        const uint64_t cut = first + (static_cast<uint64_t>(n) - first) * (c - 1) / (ranges - 1);
        split.start[c] = static_cast<uint32_t>(cut) & ~127U;
    }
    split.start[ranges] = n;
    for (uint32_t c = 0; c < ranges; ++c) {
        if (split.start[c] >= split.start[c + 1]) {
            return IdSplit{};
        }
    }
    return split;
}

bool same_split(const IdSplit& a, const IdSplit& b) {
    if (a.count != b.count) {
        return false;
    }
    for (uint32_t c = 0; c <= a.count && a.count > 1; ++c) {
        if (a.start[c] != b.start[c]) {
            return false;
        }
    }
    return true;
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

// fluid_sph.cpp:128-136.
uint32_t fluid_substeps(const sph_params& params, float delta_seconds) {
    float h = params.smoothing_radius;
    float gx = params.gravity[0];
    float gy = params.gravity[1];
    float gz = params.gravity[2];
    float gravity = std::max(std::sqrt(gx * gx + gy * gy + gz * gz), 0.1F);
    float stable = std::min(0.4F * h / std::sqrt(std::max(params.stiffness, 1.0F)), 0.25F * std::sqrt(h / gravity));
    float frame_step = std::min(std::max(delta_seconds, 0.0F), SPH_MAX_FRAME_STEP);
    auto steps = static_cast<uint32_t>(std::ceil(frame_step / std::max(stable, 1e-5F)));
    return std::clamp(steps, 1U, 8U);
}

// Smallest x >= 0 with sqrtf(x) >= v: since the correctly rounded square root
// is monotone, sqrtf(r2) >= v exactly when r2 >= this threshold.
float sqrt_at_least(float v) {
    uint32_t lo = 0;
    uint32_t hi = 0x7F800000u;  // +inf
    while (lo < hi) {
        uint32_t mid = lo + (hi - lo) / 2;
        float x;
        std::memcpy(&x, &mid, sizeof(x));
        if (std::sqrt(x) >= v) {
            hi = mid;
        } else {
            lo = mid + 1;
        }
    }
    float out;
    std::memcpy(&out, &lo, sizeof(out));
    return out;
}

// Largest x >= 0 with sqrtf(x) <= v (sqrtf(r2) <= v exactly when r2 <= it).
float sqrt_at_most(float v) {
    uint32_t lo = 0;
    uint32_t hi = 0x7F800000u;
    // Smallest x with sqrtf(x) > v, minus one.
    while (lo < hi) {
        uint32_t mid = lo + (hi - lo) / 2;
        float x;
        std::memcpy(&x, &mid, sizeof(x));
        if (std::sqrt(x) > v) {
            hi = mid;
        } else {
            lo = mid + 1;
        }
    }
    uint32_t bits = lo == 0 ? 0 : lo - 1;
    float out;
    std::memcpy(&out, &bits, sizeof(out));
    return out;
}

// The per-particle constants of fluid_sph.cpp:24-46 and :194-285, each from
// the reference's own float expression (std::pow(float, float) is powf).
TankConst make_tank_const(const sph_params& p, float dt) {
    TankConst t{};
    float h = p.smoothing_radius;
    t.h = h;
    t.h2 = h * h;
    t.c_poly6 = 315.0F / (64.0F * kPi * std::pow(h, 9.0F));
    t.c_spiky = -45.0F / (kPi * std::pow(h, 6.0F));
    t.c_visc = 45.0F / (kPi * std::pow(h, 6.0F));
    t.mass = p.gravity[3];
    t.neg_mass = -t.mass;
    t.visc_mass = p.viscosity * t.mass;
    t.rest_density = p.rest_density;
    t.stiffness = p.stiffness;
    t.dt = dt;
    t.max_speed = dt > 0.0F ? 0.4F * h / dt : 0.0F;
    // fluid_sph.cpp:245-248 skips a pair when length >= h or length <= 1e-6.
    t.r2_far = sqrt_at_least(h);
    t.r2_near = sqrt_at_most(1e-6F);
    for (int a = 0; a < 3; ++a) {
        t.gravity[a] = p.gravity[a];
        t.low[a] = p.container_min[a] + p.container_min[3];
        t.high[a] = p.container_max[a] - p.container_min[3];
        t.lattice[a] = p.lattice[a];
    }
    t.restitution = p.container_max[3];
    t.rest_w = p.rest_density;
    t.spacing = p.emitter_half_extents[3];
    t.cell_mask = p.lattice[3] - 1U;
    t.active = 1;
    std::memcpy(t.emitter_world, p.emitter_world, sizeof(t.emitter_world));
    t.radius = p.container_min[3];
    // Colliders and force fields are attached by the engine, which owns their device copies.
    t.collider_count = 0;
    t.field_count = 0;
    t.colliders = nullptr;
    t.fields = nullptr;
    return t;
}

int validate_params(const sph_params& p) {
    uint32_t cells = p.lattice[3];
    if (cells == 0 || (cells & (cells - 1)) != 0) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    if (!(p.smoothing_radius > 0.0F) || !std::isfinite(p.smoothing_radius)) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    if (p.collider_count > SPH_MAX_COLLIDERS || p.field_count > SPH_MAX_FORCE_FIELDS) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    for (uint32_t c = 0; c < p.collider_count; ++c) {
        if (p.colliders[c].type > 5) {  // scene::ColliderShape: sphere .. mesh
            return SPH_ERR_INVALID_ARGUMENT;
        }
    }
    return SPH_OK;
}

Engine::~Engine() { release(); }

int Engine::fail(cudaError_t error, const char* what) {
    last_error_ = std::string(what) + ": " + cudaGetErrorString(error);
    cudaGetLastError();
    return error == cudaErrorMemoryAllocation ? SPH_ERR_OUT_OF_MEMORY : SPH_ERR_CUDA;
}

#define SPH_CUDA(call)                                \
    do {                                              \
        cudaError_t sph_error_ = (call);              \
        if (sph_error_ != cudaSuccess) {              \
            return fail(sph_error_, #call);           \
        }                                             \
    } while (0)

template <typename T> int Engine::alloc(T** ptr, size_t count) {
    size_t bytes = std::max<size_t>(count, 1) * sizeof(T);
    SPH_CUDA(cudaMalloc(reinterpret_cast<void**>(ptr), bytes));
    device_bytes_ += bytes;
    return SPH_OK;
}

void Engine::release() {
    if (device_bytes_ == 0 && stream_ == nullptr) {
        return;
    }
    cudaSetDevice(device_);
    if (graph_ != nullptr) {
        cudaGraphExecDestroy(graph_);
        graph_ = nullptr;
    }
    drop_host_graph();
    if (learned_graph_ != nullptr) {
        cudaGraphExecDestroy(learned_graph_);
        learned_graph_ = nullptr;
    }
    for (cudaEvent_t& e : events_) {
        if (e != nullptr) {
            cudaEventDestroy(e);
            e = nullptr;
        }
    }
    for (cudaEvent_t& e : copy_events_) {
        if (e != nullptr) {
            cudaEventDestroy(e);
            e = nullptr;
        }
    }
    if (copy_stream_ != nullptr) {
        cudaStreamDestroy(copy_stream_);
        copy_stream_ = nullptr;
    }
    for (cudaEvent_t& e : range_events_) {
        if (e != nullptr) {
            cudaEventDestroy(e);
            e = nullptr;
        }
    }
    if (range_stream_ != nullptr) {
        cudaStreamDestroy(range_stream_);
        range_stream_ = nullptr;
    }
    if (flag_host_ != nullptr) {
        cudaFreeHost(flag_host_);
        flag_host_ = nullptr;
    }
    void* buffers[] = {surface_field_, surface_runs_, surface_vertices_, surface_codes_, surface_tiles_, sweep_,
                       d_tanks_,       d_colliders_,  d_fields_,    field_accel_, pos_,          vel_,         prev_,        tank_of_,   stank_,
                       grid_.keys,     grid_.keys_a,  grid_.vals_a, grid_.keys_b, grid_.vals_b, grid_.hist,
                       bucket_,        spos_,         spos2_,       svel_,        counters_,  stats_acc_,
                       bucket_stats_,  tuning_.pair_list, tuning_.pair_count, tuning_.masks,
                       rank_,          order_,        compact_ids_, compact_sorted_, compact_ranges_,
                       snap_pos_[0], snap_vel_[0],
                       snap_pos_[1],   snap_vel_[1],  sforce_,      scorrection_, sfeatures_, correction_sums_,
                       compact_rank_,  compact_order_, sx_tiles_, counts_, block_sums_, curve_ranges_};
    for (void* b : buffers) {
        if (b != nullptr) {
            cudaFree(b);
        }
    }
    if (stream_ != nullptr) {
        cudaStreamDestroy(stream_);
        stream_ = nullptr;
    }
    device_bytes_ = 0;
}

int Engine::init(int device, const std::vector<sph_params>& params, const std::vector<uint32_t>& capacities) {
    if (params.empty() || params.size() != capacities.size() || params.size() > 65535) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    for (const sph_params& p : params) {
        int status = validate_params(p);
        if (status != SPH_OK) {
            return status;
        }
    }
    int devices = 0;
    if (cudaGetDeviceCount(&devices) != cudaSuccess || devices == 0) {
        cudaGetLastError();
        last_error_ = "no CUDA device";
        return SPH_ERR_NO_DEVICE;
    }
    if (device < 0 || device >= devices) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    device_ = device;
    SPH_CUDA(cudaSetDevice(device_));
    SPH_CUDA(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));

    params_ = params;
    capacity_ = capacities;
    tanks_.resize(params.size());
    uint64_t particles = 0;
    uint64_t buckets = 0;
    for (size_t t = 0; t < params.size(); ++t) {
        tanks_[t] = make_tank_const(params[t], 0.0F);
        tanks_[t].particle_base = static_cast<uint32_t>(particles);
        tanks_[t].bucket_base = static_cast<uint32_t>(buckets);
        tanks_[t].particle_count = params.size() == 1 ? 0 : capacities[t];
        particles += capacities[t];
        buckets += params[t].lattice[3];
    }
    if (particles == 0 || particles > 0x7FFFFFFFu || buckets > 0x7FFFFFFFu) {
        return SPH_ERR_CAPACITY;
    }
    total_capacity_ = static_cast<uint32_t>(particles);
    total_buckets_ = static_cast<uint32_t>(buckets);
    curve_layout();
    total_count_ = params.size() == 1 ? 0 : total_capacity_;
    plan_ = plan_radix(bit_width(total_buckets_ - 1U), radix_bits_);

    uint32_t n = total_capacity_;
    int status = SPH_OK;
    if ((status = alloc(&d_tanks_, tanks_.size())) != SPH_OK ||
        (status = alloc(&d_colliders_, tanks_.size() * SPH_MAX_COLLIDERS)) != SPH_OK ||
        (status = alloc(&d_fields_, tanks_.size() * SPH_MAX_FORCE_FIELDS)) != SPH_OK ||
        (status = alloc(&pos_, n)) != SPH_OK ||
        (status = alloc(&vel_, n)) != SPH_OK || (status = alloc(&prev_, n)) != SPH_OK ||
        (status = alloc(&grid_.keys, n)) != SPH_OK || (status = alloc(&grid_.keys_a, n)) != SPH_OK ||
        (status = alloc(&grid_.vals_a, n)) != SPH_OK || (status = alloc(&grid_.keys_b, n)) != SPH_OK ||
        (status = alloc(&grid_.vals_b, n)) != SPH_OK ||
        (status = alloc(&grid_.hist, static_cast<size_t>(radix_tiles(n)) * kRadixMaxBins)) != SPH_OK ||
        (status = alloc(&sweep_, onesweep_scratch_words(n, kSweepMaxPasses))) != SPH_OK ||
        (status = alloc(&bucket_, total_buckets_)) != SPH_OK || (status = alloc(&spos_, n)) != SPH_OK ||
        (status = alloc(&spos2_, n)) != SPH_OK || (status = alloc(&svel_, n)) != SPH_OK ||
        (status = alloc(&counters_, 1)) != SPH_OK ||
        (status = alloc(&stats_acc_, tanks_.size() * kStatsPerTank)) != SPH_OK ||
        (status = alloc(&bucket_stats_, 2)) != SPH_OK ||
        (status = alloc(&tuning_.pair_list, static_cast<size_t>(n) * tuning_.list_cap)) != SPH_OK ||
        (status = alloc(&tuning_.pair_count, n)) != SPH_OK ||
        (status = alloc(&tuning_.masks, static_cast<size_t>(n) * 27)) != SPH_OK ||
        (status = alloc(&counts_, total_buckets_)) != SPH_OK ||
        (status = alloc(&block_sums_, counting_block_sums(total_buckets_))) != SPH_OK) {
        return status;
    }
    if ((status = alloc(&rank_, n)) != SPH_OK || (status = alloc(&order_, n)) != SPH_OK ||
        (status = alloc(&curve_ranges_, curve_capacity_ = std::min(
                                            std::max(size_t{1} << (3 * kCurveCountBits),
                                                     tanks_.size() > 1 ? static_cast<size_t>(curve_bins_) : 0),
                                            static_cast<size_t>(total_buckets_)))) != SPH_OK) {
        return status;
    }
    if (tanks_.size() > 1) {
        if ((status = alloc(&tank_of_, n)) != SPH_OK || (status = alloc(&stank_, n)) != SPH_OK) {
            return status;
        }
        std::vector<uint16_t> owner(n);
        for (size_t t = 0; t < tanks_.size(); ++t) {
            std::fill(owner.begin() + tanks_[t].particle_base,
                      owner.begin() + tanks_[t].particle_base + capacities[t], static_cast<uint16_t>(t));
        }
        SPH_CUDA(cudaMemcpy(tank_of_, owner.data(), n * sizeof(uint16_t), cudaMemcpyHostToDevice));
    }
    SPH_CUDA(cudaMemsetAsync(pos_, 0, sizeof(float4) * n, stream_));
    SPH_CUDA(cudaMemsetAsync(vel_, 0, sizeof(float4) * n, stream_));
    SPH_CUDA(cudaMemsetAsync(prev_, 0, sizeof(float4) * n, stream_));
    colliders_host_.assign(tanks_.size() * SPH_MAX_COLLIDERS, sph_collider{});
    fields_host_.assign(tanks_.size() * SPH_MAX_FORCE_FIELDS, sph_force_field{});
    for (uint32_t t = 0; t < tanks_.size(); ++t) {
        attach_shapes(t);
    }
    consts_dirty_ = true;
    shapes_dirty_ = true;
    return update_shape_flags();
}

void Engine::attach_shapes(uint32_t tank) {
    const sph_params& p = params_[tank];
    TankConst& k = tanks_[tank];
    k.collider_count = p.collider_count;
    k.field_count = p.field_count;
    k.colliders = d_colliders_ + static_cast<size_t>(tank) * SPH_MAX_COLLIDERS;
    k.fields = d_fields_ + static_cast<size_t>(tank) * SPH_MAX_FORCE_FIELDS;
    k.field_accel = field_accel_;
    std::copy(p.colliders, p.colliders + SPH_MAX_COLLIDERS,
              colliders_host_.begin() + static_cast<size_t>(tank) * SPH_MAX_COLLIDERS);
    std::copy(p.fields, p.fields + SPH_MAX_FORCE_FIELDS,
              fields_host_.begin() + static_cast<size_t>(tank) * SPH_MAX_FORCE_FIELDS);
}

int Engine::set_params(uint32_t tank, const sph_params& params) {
    if (tank >= tanks_.size()) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    int status = validate_params(params);
    if (status != SPH_OK) {
        return status;
    }
    if (params.lattice[3] != params_[tank].lattice[3]) {
        // The bucket table is laid out at create; a new bucket count needs a new context.
        return SPH_ERR_CAPACITY;
    }
    TankConst fresh = make_tank_const(params, tanks_[tank].dt);
    fresh.particle_base = tanks_[tank].particle_base;
    fresh.bucket_base = tanks_[tank].bucket_base;
    fresh.particle_count = tanks_[tank].particle_count;
    fresh.active = tanks_[tank].active;
    tanks_[tank] = fresh;
    params_[tank] = params;
    attach_shapes(tank);
    consts_dirty_ = true;
    shapes_dirty_ = true;
    return update_shape_flags();
}

int Engine::update_shape_flags() {
    bool fields = false;
    bool colliders = false;
    for (const TankConst& t : tanks_) {
        fields = fields || t.field_count != 0;
        colliders = colliders || t.collider_count != 0;
    }
    if (fields && field_accel_ == nullptr) {
        int status = alloc(&field_accel_, total_capacity_);
        if (status != SPH_OK) {
            return status;
        }
        for (TankConst& t : tanks_) {
            t.field_accel = field_accel_;
        }
    }
    if (fields != has_fields_ || colliders != has_colliders_) {
        // The substep's launch list changes: capture the graphs again.
        if (graph_ != nullptr) {
            cudaGraphExecDestroy(graph_);
            graph_ = nullptr;
        }
        drop_host_graph();
        if (learned_graph_ != nullptr) {
            cudaGraphExecDestroy(learned_graph_);
            learned_graph_ = nullptr;
        }
    }
    has_fields_ = fields;
    has_colliders_ = colliders;
    return SPH_OK;
}

int Engine::enqueue_fields(uint32_t* launches) {
    if (has_fields_) {
        SPH_CUDA(launch_fields(pos_, tank_of_, d_tanks_, total_count_, field_accel_, stream_));
        if (launches != nullptr) {
            *launches += 1;
        }
    }
    return SPH_OK;
}

int Engine::enqueue_colliders(uint32_t* launches) {
    if (has_colliders_) {
        SPH_CUDA(launch_colliders(pos_, vel_, tank_of_, d_tanks_, total_count_, stream_));
        if (launches != nullptr) {
            *launches += 1;
        }
    }
    return SPH_OK;
}

int Engine::refresh_constants(float dt) {
    if (!consts_dirty_ && dt == const_dt_) {
        if (active_dirty_) {
            // A new active mask alone: patch the flags of the device table.
            active_host_.resize(tanks_.size());
            for (size_t t = 0; t < tanks_.size(); ++t) {
                active_host_[t] = static_cast<uint8_t>(tanks_[t].active);
            }
            SPH_CUDA(launch_set_active(d_tanks_, active_host_.data(), static_cast<uint32_t>(tanks_.size()), stream_));
            active_dirty_ = false;
        }
        return SPH_OK;
    }
    active_dirty_ = false;  // the whole table goes up below
    for (TankConst& t : tanks_) {
        t.dt = dt;
        t.max_speed = dt > 0.0F ? 0.4F * t.h / dt : 0.0F;
    }
    curve_layout();
    SPH_CUDA(cudaMemcpyAsync(d_tanks_, tanks_.data(), tanks_.size() * sizeof(TankConst), cudaMemcpyHostToDevice,
                             stream_));
    if (shapes_dirty_) {
        SPH_CUDA(cudaMemcpyAsync(d_colliders_, colliders_host_.data(), colliders_host_.size() * sizeof(sph_collider),
                                 cudaMemcpyHostToDevice, stream_));
        SPH_CUDA(cudaMemcpyAsync(d_fields_, fields_host_.data(), fields_host_.size() * sizeof(sph_force_field),
                                 cudaMemcpyHostToDevice, stream_));
    }
    const_dt_ = dt;
    consts_dirty_ = false;
    shapes_dirty_ = false;
    return SPH_OK;
}

int Engine::upload(uint32_t tank, const float* pos, const float* vel, uint32_t count) {
    if (tank >= tanks_.size() || (count > 0 && pos == nullptr)) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    if (count > capacity_[tank] || (tanks_.size() > 1 && count != capacity_[tank])) {
        return SPH_ERR_CAPACITY;
    }
    SPH_CUDA(cudaSetDevice(device_));
    uint32_t base = tanks_[tank].particle_base;
    size_t bytes = sizeof(float4) * count;
    if (count > 0) {
        SPH_CUDA(cudaMemcpyAsync(pos_ + base, pos, bytes, cudaMemcpyHostToDevice, stream_));
        if (vel != nullptr) {
            SPH_CUDA(cudaMemcpyAsync(vel_ + base, vel, bytes, cudaMemcpyHostToDevice, stream_));
        } else {
            SPH_CUDA(cudaMemsetAsync(vel_ + base, 0, bytes, stream_));
        }
        SPH_CUDA(cudaMemcpyAsync(prev_ + base, pos_ + base, bytes, cudaMemcpyDeviceToDevice, stream_));
        // Non-finite xyz in either array is rejected (checked on the device,
        // where the data already is).
        SPH_CUDA(cudaMemsetAsync(bucket_stats_, 0, sizeof(uint32_t), stream_));
        SPH_CUDA(launch_count_nonfinite(pos_ + base, vel_ + base, count, bucket_stats_, stream_));
        SPH_CUDA(cudaMemcpyAsync(&nonfinite_host_, bucket_stats_, sizeof(uint32_t), cudaMemcpyDeviceToHost, stream_));
    } else {
        nonfinite_host_ = 0;
    }
    SPH_CUDA(cudaStreamSynchronize(stream_));
    if (nonfinite_host_ != 0) {
        return SPH_ERR_NONFINITE;
    }
    if (tanks_.size() == 1 && (tanks_[0].particle_count != count || total_count_ != count)) {
        tanks_[0].particle_count = count;
        total_count_ = count;
        consts_dirty_ = true;  // the device tank table carries the count
    }
    grid_valid_ = false;
    return SPH_OK;
}

int Engine::download(uint32_t tank, float* pos, float* vel) {
    if (tank >= tanks_.size()) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    SPH_CUDA(cudaSetDevice(device_));
    SPH_CUDA(cudaStreamSynchronize(stream_));
    uint32_t base = tanks_[tank].particle_base;
    size_t bytes = sizeof(float4) * tanks_[tank].particle_count;
    if (bytes == 0) {
        return SPH_OK;
    }
    if (pos != nullptr) {
        SPH_CUDA(cudaMemcpy(pos, pos_ + base, bytes, cudaMemcpyDeviceToHost));
    }
    if (vel != nullptr) {
        SPH_CUDA(cudaMemcpy(vel, vel_ + base, bytes, cudaMemcpyDeviceToHost));
    }
    return SPH_OK;
}

int Engine::step_host(const float* pos_in, const float* vel_in, uint32_t count, float dt, uint32_t substeps,
                      float* pos_out, float* vel_out) {
    if (tanks_.size() != 1 || (count > 0 && pos_in == nullptr) || !(dt > 0.0F) || !std::isfinite(dt)) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    if (count > capacity_[0]) {
        return SPH_ERR_CAPACITY;
    }
    if (count == 0 || substeps == 0) {  // nothing to overlap
        int status = upload(0, pos_in, vel_in, count);
        if (status == SPH_OK) {
            status = run(dt, substeps);
        }
        return status == SPH_OK ? download(0, pos_out, vel_out) : status;
    }
    SPH_CUDA(cudaSetDevice(device_));
    if (copy_stream_ == nullptr) {
        SPH_CUDA(cudaStreamCreateWithFlags(&copy_stream_, cudaStreamNonBlocking));
        SPH_CUDA(cudaStreamCreateWithFlags(&range_stream_, cudaStreamNonBlocking));
        for (cudaEvent_t& e : copy_events_) {
            SPH_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        }
        for (cudaEvent_t& e : range_events_) {
            SPH_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        }
        SPH_CUDA(cudaMallocHost(&flag_host_, sizeof(uint32_t)));
    }
    if (tanks_[0].particle_count != count || total_count_ != count) {
        tanks_[0].particle_count = count;
        total_count_ = count;
        consts_dirty_ = true;  // the device tank table carries the count
    }
    int status = refresh_constants(dt);
    if (status != SPH_OK) {
        return status;
    }
    // The overlapped form: one tank in a curve order, the mask kernels, no
    // colliders (they move particles of every id range after integrate).
    const bool overlap = tanks_.size() == 1 && schedule_curve_ != 0 && tuning_.variant == 4 && !has_colliders_ &&
                         count >= kHostOverlapMin;
    want_ranges_ = overlap ? kHostRanges : 0;
    // Positions first: the grid reads nothing else. The velocities follow on
    // the copy stream, with upload's keepRendered copy and the non-finite
    // check of both arrays, while the grid is built. In the overlapped form
    // the first gather leaves the velocities out and the copy stream gathers
    // them beside the density pass (which writes only the pressure word of
    // each sorted velocity).
    const size_t bytes = sizeof(float4) * count;
    SPH_CUDA(cudaMemcpyAsync(pos_, pos_in, bytes, cudaMemcpyHostToDevice, stream_));
    SPH_CUDA(cudaEventRecord(copy_events_[0], stream_));
    SPH_CUDA(cudaStreamWaitEvent(copy_stream_, copy_events_[0], 0));
    if (vel_in != nullptr) {
        SPH_CUDA(cudaMemcpyAsync(vel_, vel_in, bytes, cudaMemcpyHostToDevice, copy_stream_));
    } else {
        SPH_CUDA(cudaMemsetAsync(vel_, 0, bytes, copy_stream_));
    }
    SPH_CUDA(cudaMemcpyAsync(prev_, pos_, bytes, cudaMemcpyDeviceToDevice, copy_stream_));
    SPH_CUDA(cudaMemsetAsync(bucket_stats_, 0, sizeof(uint32_t), copy_stream_));
    SPH_CUDA(launch_count_nonfinite(pos_, vel_, count, bucket_stats_, copy_stream_));
    SPH_CUDA(cudaMemcpyAsync(flag_host_, bucket_stats_, sizeof(uint32_t), cudaMemcpyDeviceToHost, copy_stream_));
    SPH_CUDA(cudaEventRecord(copy_events_[1], copy_stream_));
    if (overlap && substeps == 1) {
        // The one-substep form from a graph (the order remade beforehand
        // when due; the capture holds only its scatter).
        if ((status = prepare_schedule(nullptr)) != SPH_OK || (status = ensure_host_graph()) != SPH_OK) {
            return status;
        }
        SPH_CUDA(cudaGraphLaunch(host_graph_, stream_));
    } else if (overlap) {
        defer_vel_ = true;
        status = enqueue_grid(nullptr);
        defer_vel_ = false;
        if (status != SPH_OK) {
            return status;
        }
        // The copy stream: sorted ids ready -> velocities gathered. Integrate
        // waits for it, and so for the check before it (integrate rewrites
        // the arrays the check and the keepRendered copy read).
        SPH_CUDA(cudaEventRecord(copy_events_[2], stream_));
        SPH_CUDA(cudaStreamWaitEvent(copy_stream_, copy_events_[2], 0));
        SPH_CUDA(launch_gather_vel(grid_.sorted_ids, count, vel_, svel_, copy_stream_));
        SPH_CUDA(cudaEventRecord(copy_events_[3], copy_stream_));
        if ((status = enqueue_fields(nullptr)) != SPH_OK) {
            return status;
        }
        SPH_CUDA(launch_density(spos_, svel_, spos2_, bucket_, d_tanks_, stank_, count, nullptr, stream_, tuning_));
        SPH_CUDA(cudaStreamWaitEvent(stream_, copy_events_[3], 0));
        SPH_CUDA(launch_integrate(spos2_, svel_, grid_.sorted_ids, bucket_, d_tanks_, stank_, count, pos_, vel_,
                                  stream_, tuning_));
    } else {
        // The first substep launched directly, its gather waiting for the
        // copy stream; the rest through the graph, as run() does.
        gather_wait_ = copy_events_[1];
        status = enqueue_substep(nullptr);
        gather_wait_ = nullptr;
    }
    if (status != SPH_OK) {
        return status;
    }
    if (substeps > 1) {
        if ((status = ensure_graph()) != SPH_OK) {
            return status;
        }
        const uint32_t graphed = overlap ? substeps - 1 : substeps;
        for (uint32_t s = 1; s < graphed; ++s) {
            if ((status = prepare_schedule(nullptr)) != SPH_OK) {
                return status;
            }
            SPH_CUDA(cudaGraphLaunch(graph_, stream_));
        }
        if (overlap) {  // the last substep direct, its integrate in id ranges
            if ((status = enqueue_grid(nullptr)) != SPH_OK || (status = enqueue_fields(nullptr)) != SPH_OK) {
                return status;
            }
            SPH_CUDA(
                launch_density(spos_, svel_, spos2_, bucket_, d_tanks_, stank_, count, nullptr, stream_, tuning_));
            if ((status = enqueue_integrate_ranges()) != SPH_OK) {
                return status;
            }
        }
    }
    grid_valid_ = true;
    // The check lands long before the substeps end: read it then, and queue
    // the download behind them so that it starts as the last pass ends (in
    // the overlapped form, each id range's rows as soon as they are
    // integrated).
    SPH_CUDA(cudaEventSynchronize(copy_events_[1]));
    if (*flag_host_ != 0) {
        SPH_CUDA(cudaStreamSynchronize(stream_));
        return SPH_ERR_NONFINITE;  // the caller's arrays are left as they were
    }
    if (overlap) {
        const uint32_t ranges = rank_split_.count > 1 ? rank_split_.count : 1U;
        for (uint32_t c = 0; c < ranges; ++c) {
            const size_t first = ranges > 1 ? rank_split_.start[c] : 0;
            const size_t rows = (ranges > 1 ? rank_split_.start[c + 1] : count) - first;
            SPH_CUDA(cudaStreamWaitEvent(copy_stream_, copy_events_[4 + c], 0));
            if (pos_out != nullptr) {
                SPH_CUDA(cudaMemcpyAsync(pos_out + 4 * first, pos_ + first, sizeof(float4) * rows,
                                         cudaMemcpyDeviceToHost, copy_stream_));
            }
            if (vel_out != nullptr) {
                SPH_CUDA(cudaMemcpyAsync(vel_out + 4 * first, vel_ + first, sizeof(float4) * rows,
                                         cudaMemcpyDeviceToHost, copy_stream_));
            }
        }
        SPH_CUDA(cudaStreamSynchronize(copy_stream_));
    } else {
        if (pos_out != nullptr) {
            SPH_CUDA(cudaMemcpyAsync(pos_out, pos_, bytes, cudaMemcpyDeviceToHost, stream_));
        }
        if (vel_out != nullptr) {
            SPH_CUDA(cudaMemcpyAsync(vel_out, vel_, bytes, cudaMemcpyDeviceToHost, stream_));
        }
    }
    SPH_CUDA(cudaStreamSynchronize(stream_));
    return SPH_OK;
}

// The integrate pass over the id ranges of the processing order, an event
// after each (step_host downloads range c's rows once its event fires).
// Range c + 1 is a programmatic dependent of range c (ranges write disjoint
// rows and read only what density wrote), so its blocks start as range c's
// last blocks leave the SMs, where a plain second launch would wait for
// range c's slowest block. Range c's event is recorded on range_stream_
// after a plain wait for range c, which also joins stream_ again after the
// last range. Without ranges in the order: one whole pass, one event.
// While capturing, the range events become the graph's external records.
int Engine::enqueue_integrate_ranges() {
    const uint32_t n = total_count_;
    const uint32_t ranges = rank_split_.count > 1 && schedule_curve_ != 0 ? rank_split_.count : 1U;
    const unsigned int record = capturing_ ? cudaEventRecordExternal : cudaEventRecordDefault;
    NeighbourTuning t = tuning_;
    for (uint32_t c = 0; c < ranges; ++c) {
        if (ranges > 1) {
            t.slot_begin = rank_split_.start[c];
            t.slot_end = rank_split_.start[c + 1];
            t.programmatic = c > 0;
        }
        SPH_CUDA(launch_integrate(spos2_, svel_, grid_.sorted_ids, bucket_, d_tanks_, stank_, n, pos_, vel_, stream_,
                                  t));
        if (ranges == 1) {
            SPH_CUDA(cudaEventRecordWithFlags(copy_events_[4], stream_, record));
        } else {
            SPH_CUDA(cudaEventRecord(range_events_[0], stream_));
            SPH_CUDA(cudaStreamWaitEvent(range_stream_, range_events_[0], 0));
            SPH_CUDA(cudaEventRecordWithFlags(copy_events_[4 + c], range_stream_, record));
        }
    }
    if (ranges > 1) {
        SPH_CUDA(cudaEventRecord(range_events_[1], range_stream_));
        SPH_CUDA(cudaStreamWaitEvent(stream_, range_events_[1], 0));
    }
    return SPH_OK;
}

void Engine::drop_host_graph() {
    if (host_graph_ != nullptr) {
        cudaGraphExecDestroy(host_graph_);
        host_graph_ = nullptr;
    }
}

// step_host's one-substep overlapped form as a graph on stream_: the grid
// (its gather without velocities), the velocity gather on the copy stream once
// the ids are sorted and the upload is checked (events[1], recorded outside),
// density beside it, then integrate by id ranges with an external event after
// each. Captured again when the count, the order's id ranges or the launch
// shape change.
int Engine::ensure_host_graph() {
    if (host_graph_ != nullptr && host_graph_count_ == total_count_ && same_split(host_graph_split_, rank_split_)) {
        return SPH_OK;
    }
    drop_host_graph();
    const uint32_t n = total_count_;
    cudaGraph_t graph = nullptr;
    SPH_CUDA(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
    capturing_ = true;
    defer_vel_ = true;
    int status = enqueue_grid(nullptr);
    defer_vel_ = false;
    cudaError_t err = cudaSuccess;
    if (status == SPH_OK) {
        err = cudaEventRecord(copy_events_[2], stream_);
        if (err == cudaSuccess) {
            err = cudaStreamWaitEvent(copy_stream_, copy_events_[2], 0);  // the copy stream joins the capture
        }
        if (err == cudaSuccess) {
            err = cudaStreamWaitEvent(copy_stream_, copy_events_[1], cudaEventWaitExternal);
        }
        if (err == cudaSuccess) {
            err = launch_gather_vel(grid_.sorted_ids, n, vel_, svel_, copy_stream_);
        }
        if (err == cudaSuccess) {
            err = cudaEventRecord(copy_events_[3], copy_stream_);
        }
    }
    if (status == SPH_OK && err == cudaSuccess) {
        status = enqueue_fields(nullptr);
    }
    if (status == SPH_OK && err == cudaSuccess) {
        err = launch_density(spos_, svel_, spos2_, bucket_, d_tanks_, stank_, n, nullptr, stream_, tuning_);
        if (err == cudaSuccess) {
            err = cudaStreamWaitEvent(stream_, copy_events_[3], 0);  // and rejoins it
        }
    }
    if (status == SPH_OK && err == cudaSuccess) {
        status = enqueue_integrate_ranges();
    }
    capturing_ = false;
    const cudaError_t end = cudaStreamEndCapture(stream_, &graph);
    if (status == SPH_OK && err == cudaSuccess) {
        err = end;
    }
    if (err == cudaSuccess && status == SPH_OK) {
        err = cudaGraphInstantiate(&host_graph_, graph, 0);
    }
    if (graph != nullptr) {
        cudaGraphDestroy(graph);
    }
    if (status != SPH_OK) {
        return status;
    }
    if (err != cudaSuccess) {
        host_graph_ = nullptr;
        return fail(err, "step_host graph");
    }
    host_graph_count_ = n;
    host_graph_split_ = rank_split_;
    return SPH_OK;
}

int Engine::download_previous(uint32_t tank, float* pos) {
    if (tank >= tanks_.size() || pos == nullptr) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    SPH_CUDA(cudaSetDevice(device_));
    SPH_CUDA(cudaStreamSynchronize(stream_));
    size_t bytes = sizeof(float4) * tanks_[tank].particle_count;
    if (bytes > 0) {
        SPH_CUDA(cudaMemcpy(pos, prev_ + tanks_[tank].particle_base, bytes, cudaMemcpyDeviceToHost));
    }
    return SPH_OK;
}

int Engine::keep_rendered() {
    SPH_CUDA(cudaSetDevice(device_));
    if (total_count_ > 0) {
        SPH_CUDA(cudaMemcpyAsync(prev_, pos_, sizeof(float4) * total_count_, cudaMemcpyDeviceToDevice, stream_));
    }
    return SPH_OK;
}

int Engine::write_instances(sph_instance* instances, uint32_t instance_base, uint32_t sphere_mesh,
                            sph_tlas_instance* tlas, uint32_t tlas_base, uint64_t blas, uint32_t fluid_index,
                            uint32_t flags) {
    if (instances == nullptr || ((flags & SPH_INSTANCES_WRITE_TLAS) != 0 && tlas == nullptr) ||
        reinterpret_cast<uintptr_t>(instances) % 16 != 0 || reinterpret_cast<uintptr_t>(tlas) % 16 != 0 ||
        (flags & ~(SPH_INSTANCES_RESET_HISTORY | SPH_INSTANCES_WRITE_TLAS | SPH_INSTANCES_SURFACE_TLAS)) != 0) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    SPH_CUDA(cudaSetDevice(device_));
    const uint32_t n = tanks_[0].particle_count;
    SPH_CUDA(launch_instances(pos_, prev_, n, params_[0].container_min[3], instances, instance_base, sphere_mesh,
                              (flags & SPH_INSTANCES_WRITE_TLAS) != 0 ? tlas : nullptr, tlas_base, blas, fluid_index,
                              flags, stream_));
    // The kernel has kept particles [0, n); tanks behind the first keep theirs here.
    if (total_count_ > n) {
        SPH_CUDA(cudaMemcpyAsync(prev_ + n, pos_ + n, sizeof(float4) * (total_count_ - n), cudaMemcpyDeviceToDevice,
                                 stream_));
    }
    return SPH_OK;
}

int Engine::emit(uint32_t tank, uint32_t count) {
    if (tank >= tanks_.size()) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    if (count > capacity_[tank] || (tanks_.size() > 1 && count != capacity_[tank])) {
        return SPH_ERR_CAPACITY;
    }
    SPH_CUDA(cudaSetDevice(device_));
    if (tanks_.size() == 1) {
        tanks_[0].particle_count = count;
        total_count_ = count;
        consts_dirty_ = true;
    }
    int status = refresh_constants(const_dt_ < 0.0F ? 0.0F : const_dt_);
    if (status != SPH_OK) {
        return status;
    }
    SPH_CUDA(launch_emit(d_tanks_ + tank, tanks_[tank].particle_base, count, pos_, vel_, prev_, stream_));
    grid_valid_ = false;
    since_refresh_ = kScheduleRefresh;  // a new lattice: remake the order at the next build
    return SPH_OK;
}

// A batch's processing order lays each tank's cells out in row order, tank
// after tank: curve_dims = the cells a side from the tank's low corner (as the
// order's kernel finds a particle's cell, clamped to them), curve_base = the
// cells of the tanks before it.
void Engine::curve_layout() {
    uint64_t bins = 0;
    for (TankConst& t : tanks_) {
        uint64_t cells = 1;
        for (int a = 0; a < 3; ++a) {
            uint32_t d = 1;
            if (t.h > 0.0F && std::isfinite(t.low[a] / t.h) && std::isfinite(t.high[a] / t.h)) {
                const double lo = std::floor(static_cast<double>(t.low[a] / t.h));
                const double hi = std::floor(static_cast<double>(t.high[a] / t.h));
                d = hi >= lo ? static_cast<uint32_t>(std::min(hi - lo + 1.0, 4096.0)) : 1U;
            }
            t.curve_dims[a] = d;
            cells *= d;
        }
        t.curve_base = bins <= 0xFFFFFFFFull ? static_cast<uint32_t>(bins) : 0U;
        bins += cells;
    }
    curve_bins_ = bins;
}

// Morton (or Hilbert) processing order: rank_ is refreshed from the current positions
// every kScheduleRefresh grid builds, kCountingRefresh when one tank's order
// is made by counting (particles move a fraction of a cell per substep, so an
// order a few substeps old keeps its locality; a fresher one runs the
// neighbour passes faster, the counting form is cheap enough to pay for that), after an emit
// and whenever the particle count changed since the last refresh. An upload or
// a restore of the same count keeps the order (still a permutation of the
// ids; the usual refresh renews its locality). Never called while a graph
// is being captured: the graphs only hold the per-substep order scatter.
int Engine::prepare_schedule(uint32_t* launches) {
    if (schedule_curve_ == 0 || total_count_ == 0) {
        return SPH_OK;
    }
    uint32_t axis_bits = 0;
    uint32_t key_bits = 0;
    schedule_bits(&axis_bits, &key_bits);
    IdSplit split = host_split(total_count_, want_ranges_);
    if (key_bits + bit_width(split.count > 1 ? split.count - 1U : 0U) > 32) {
        split = IdSplit{};
    }
    // One tank without id ranges whose whole cells fit the bins (at most
    // kCurveCountBits an axis, and within the grid's count scratch): group
    // the particles by cell with one atomic each. Else sort the curve keys
    // (grouping several cells a bin loses the locality the order is for).
    const bool by_counting = counting_curve_ && tanks_.size() == 1 && split.count <= 1 &&
                             axis_bits <= kCurveCountBits && (size_t{1} << (3 * axis_bits)) <= total_buckets_;
    const uint32_t count_bits = axis_bits;
    // A batch: the tanks' cells in row order, when they fit the bins.
    const bool batch_counting = counting_curve_ && tanks_.size() > 1 && split.count <= 1 && curve_bins_ > 0 &&
                                curve_bins_ <= curve_capacity_ && curve_bins_ <= total_buckets_;
    // Wanted id ranges that the order lacks force a remake; ranges no longer
    // wanted leave with the next regular refresh.
    if (rank_count_ == total_count_ &&
        since_refresh_ + 1 < (by_counting || batch_counting ? kCountingRefresh : kScheduleRefresh) &&
        (want_ranges_ == 0 || same_split(rank_split_, split))) {
        ++since_refresh_;
        return SPH_OK;
    }
    uint32_t made = 0;
    if (batch_counting) {
        SPH_CUDA(launch_tank_cells_rank(pos_, tank_of_, d_tanks_, total_count_, static_cast<uint32_t>(curve_bins_),
                                        grid_.keys_a, grid_.vals_a, counts_, block_sums_, curve_ranges_, rank_, stream_,
                                        &made));
    } else if (by_counting) {
        SPH_CUDA(launch_curve_rank_counting(pos_, d_tanks_, total_count_, axis_bits, axis_bits - count_bits,
                                            schedule_curve_ == 2, grid_.keys_a, grid_.vals_a, counts_, block_sums_,
                                            curve_ranges_, rank_, stream_, &made));
    } else {
        SPH_CUDA(launch_morton_rank(pos_, tank_of_, d_tanks_, total_count_, axis_bits, key_bits, grid_, sweep_,
                                    rank_, stream_, &made, schedule_curve_ == 2, nullptr, split));
    }
    kernels_launched_ += made;
    if (launches != nullptr) {
        *launches += made;
    }
    rank_count_ = total_count_;
    rank_split_ = split;
    since_refresh_ = 0;
    return SPH_OK;
}

// Bits per axis of the curve keys: enough for the widest tank's cells,
// within 32 key bits with the tank index above them.
void Engine::schedule_bits(uint32_t* axis_bits, uint32_t* key_bits) const {
    uint32_t cells = 1;
    for (const TankConst& t : tanks_) {
        for (int a = 0; a < 3; ++a) {
            float extent = (t.high[a] - t.low[a]) / t.h;
            uint32_t c = std::isfinite(extent) && extent > 0.0F ? static_cast<uint32_t>(std::min(extent, 4096.0F)) + 1U
                                                               : 1U;
            cells = std::max(cells, c);
        }
    }
    const uint32_t tank_bits = bit_width(static_cast<uint32_t>(tanks_.size()) - 1U);
    *axis_bits = std::max(1U, std::min({bit_width(cells - 1U), 10U, (32U - tank_bits) / 3U}));
    *key_bits = 3U * *axis_bits + tank_bits;
}

int Engine::enqueue_grid(uint32_t* launches) {
    uint32_t n = total_count_;
    if (!capturing_) {
        int status = prepare_schedule(nullptr);
        if (status != SPH_OK) {
            return status;
        }
    }
    if (counting_) {
        // Every bucket's range comes out of the count scan: no table clear.
        SPH_CUDA(launch_counting_grid(pos_, tank_of_, d_tanks_, n, total_buckets_, grid_, counts_, block_sums_, bucket_,
                                      stream_, launches));
    } else if (onesweep_) {
        SPH_CUDA(cudaMemsetAsync(bucket_, 0, sizeof(uint2) * total_buckets_, stream_));
        const uint32_t passes = onesweep_passes(bit_width(total_buckets_ - 1U));
        SPH_CUDA(launch_keys_onesweep(pos_, tank_of_, d_tanks_, n, grid_.keys, passes, sweep_, stream_));
        SPH_CUDA(launch_onesweep_sort(grid_, n, passes, sweep_, stream_, launches));
    } else {
        SPH_CUDA(cudaMemsetAsync(bucket_, 0, sizeof(uint2) * total_buckets_, stream_));
        SPH_CUDA(launch_keys(pos_, tank_of_, d_tanks_, n, grid_.keys, stream_));
        SPH_CUDA(launch_radix_sort(grid_, n, plan_, stream_, launches));
    }
    if (gather_wait_ != nullptr) {  // the gather is the first pass that reads velocities
        SPH_CUDA(cudaStreamWaitEvent(stream_, gather_wait_, 0));
    }
    int status = enqueue_bounds(launches);
    if (status != SPH_OK) {
        return status;
    }
    if (launches != nullptr) {
        *launches += 1;
    }
    return SPH_OK;
}

int Engine::enqueue_bounds(uint32_t* launches) {
    uint32_t n = total_count_;
    Schedule schedule{};
    if (schedule_curve_ != 0) {
        if (rank_count_ != n) {
            return SPH_ERR_INVALID_ARGUMENT;  // prepare_schedule did not run for this particle count
        }
        schedule.rank = rank_;
        schedule.order = order_;
    }
    const float4* vel = defer_vel_ ? nullptr : vel_;  // else step_host gathers them beside the density pass
    if (counting_) {
        SPH_CUDA(launch_order_gather(grid_, n, bucket_, counts_, pos_, vel, tank_of_, spos_, svel_, stank_, schedule,
                                     stream_));
    } else {
        SPH_CUDA(launch_bounds_gather(grid_.sorted_keys, grid_.sorted_ids, n, bucket_, pos_, vel, tank_of_, spos_,
                                      svel_, stank_, schedule, stream_));
    }
    tuning_.order = schedule_curve_ != 0 ? order_ : nullptr;
    if (launches != nullptr) {
        *launches += 1;
    }
    return SPH_OK;
}

int Engine::enqueue_substep(uint32_t* launches) {
    int status = enqueue_grid(launches);
    if (status != SPH_OK) {
        return status;
    }
    uint32_t n = total_count_;
    if ((status = enqueue_fields(launches)) != SPH_OK) {
        return status;
    }
    SPH_CUDA(launch_density(spos_, svel_, spos2_, bucket_, d_tanks_, stank_, n, nullptr, stream_, tuning_));
    SPH_CUDA(launch_integrate(spos2_, svel_, grid_.sorted_ids, bucket_, d_tanks_, stank_, n, pos_, vel_, stream_,
                                  tuning_));
    if (launches != nullptr) {
        *launches += 2;
    }
    return enqueue_colliders(launches);
}

int Engine::ensure_graph() {
    if (graph_ != nullptr && graph_count_ == total_count_) {
        return SPH_OK;
    }
    if (graph_ != nullptr) {
        cudaGraphExecDestroy(graph_);
        graph_ = nullptr;
    }
    drop_host_graph();
    int status = prepare_schedule(nullptr);
    if (status != SPH_OK) {
        return status;
    }
    SPH_CUDA(prepare_staged_integrate());
    cudaGraph_t graph = nullptr;
    SPH_CUDA(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
    uint32_t launches = 0;
    capturing_ = true;
    status = enqueue_substep(&launches);
    capturing_ = false;
    cudaError_t end = cudaStreamEndCapture(stream_, &graph);
    if (status != SPH_OK) {
        if (graph != nullptr) {
            cudaGraphDestroy(graph);
        }
        return status;
    }
    if (end != cudaSuccess) {
        return fail(end, "cudaStreamEndCapture");
    }
    cudaError_t inst = cudaGraphInstantiate(&graph_, graph, 0);
    cudaGraphDestroy(graph);
    if (inst != cudaSuccess) {
        graph_ = nullptr;
        return fail(inst, "cudaGraphInstantiate");
    }
    graph_count_ = total_count_;
    launches_per_substep_ = launches;
    return SPH_OK;
}

int Engine::run(float dt, uint32_t substeps) {
    if (!(dt > 0.0F) || !std::isfinite(dt)) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    if (total_count_ == 0 || substeps == 0) {
        return SPH_OK;
    }
    SPH_CUDA(cudaSetDevice(device_));
    want_ranges_ = 0;  // the next regular refresh drops step_host's id ranges
    int status = refresh_constants(dt);
    if (status != SPH_OK) {
        return status;
    }
    // A batch with most particles in tanks that sit out: build the grid over
    // the active tanks' particles only.
    if (tanks_.size() > 1 && onesweep_) {
        uint32_t active = 0;
        for (const TankConst& t : tanks_) {
            active += t.active != 0 ? t.particle_count : 0U;
        }
        if (2ull * active <= total_count_) {
            return run_compact(substeps, active);
        }
    }
    status = ensure_graph();
    if (status != SPH_OK) {
        return status;
    }
    for (uint32_t s = 0; s < substeps; ++s) {
        if ((status = prepare_schedule(nullptr)) != SPH_OK) {
            return status;
        }
        SPH_CUDA(cudaGraphLaunch(graph_, stream_));
        kernels_launched_ += launches_per_substep_;
    }
    grid_valid_ = true;
    return SPH_OK;
}

// The substep over a compacted particle set: the active tanks' ids in one
// list, keys, sort, bounds and the neighbour passes over that list only, the
// results written back through the ids. Every active particle sees exactly
// the pairs and order of a full build (tanks never share buckets), so the
// bits are the same; direct launches (the set changes between calls).
int Engine::run_compact(uint32_t substeps, uint32_t active_particles) {
    int status = SPH_OK;
    if (compact_ids_ == nullptr) {
        if ((status = alloc(&compact_ids_, total_capacity_)) != SPH_OK ||
            (status = alloc(&compact_sorted_, total_capacity_)) != SPH_OK ||
            (status = alloc(&compact_ranges_, 3 * tanks_.size())) != SPH_OK) {
            return status;
        }
    }
    compact_ranges_host_.clear();
    uint32_t compact = 0;
    for (const TankConst& t : tanks_) {
        if (t.active != 0 && t.particle_count > 0) {
            compact_ranges_host_.insert(compact_ranges_host_.end(), {t.particle_base, compact, t.particle_count});
            compact += t.particle_count;
        }
    }
    const uint32_t ranges = static_cast<uint32_t>(compact_ranges_host_.size() / 3);
    grid_valid_ = false;  // the grid buffers now hold the compacted build
    if (active_particles == 0 || ranges == 0) {
        return SPH_OK;
    }
    SPH_CUDA(cudaMemcpyAsync(compact_ranges_, compact_ranges_host_.data(), compact_ranges_host_.size() * sizeof(uint32_t),
                             cudaMemcpyHostToDevice, stream_));
    SPH_CUDA(launch_compact_ids(compact_ranges_, ranges, compact_ids_, stream_));
    const uint32_t n = active_particles;
    const uint32_t passes = onesweep_passes(bit_width(total_buckets_ - 1U));
    NeighbourTuning tuning = tuning_;
    tuning.order = nullptr;
    // Bucket runs (first bucket, count) of adjacent active tanks.
    std::vector<uint2> clear_runs;
    for (const TankConst& t : tanks_) {
        if (t.active == 0 || t.particle_count == 0) {
            continue;
        }
        const uint32_t count = t.cell_mask + 1U;
        if (!clear_runs.empty() && clear_runs.back().x + clear_runs.back().y == t.bucket_base) {
            clear_runs.back().y += count;
        } else {
            clear_runs.push_back(make_uint2(t.bucket_base, count));
        }
    }
    // The compacted set gets its own processing order (made once per call,
    // in buffers of its own, so the full set's order stays valid).
    Schedule schedule{};
    if (schedule_curve_ != 0) {
        if (compact_rank_ == nullptr) {
            if ((status = alloc(&compact_rank_, total_capacity_)) != SPH_OK ||
                (status = alloc(&compact_order_, total_capacity_)) != SPH_OK) {
                return status;
            }
        }
        uint32_t axis_bits = 0;
        uint32_t key_bits = 0;
        schedule_bits(&axis_bits, &key_bits);
        SPH_CUDA(launch_morton_rank(pos_, tank_of_, d_tanks_, n, axis_bits, key_bits, grid_, sweep_, compact_rank_,
                                    stream_, nullptr, schedule_curve_ == 2, compact_ids_));
        schedule.rank = compact_rank_;
        schedule.order = compact_order_;
        tuning.order = compact_order_;
    }
    for (uint32_t s = 0; s < substeps; ++s) {
        // Only the active tanks' buckets are read, so only they need clearing:
        // one memset per run of adjacent active tanks while that is the
        // smaller job.
        if (clear_runs.size() <= 32) {
            for (const uint2& r : clear_runs) {
                SPH_CUDA(cudaMemsetAsync(bucket_ + r.x, 0, sizeof(uint2) * r.y, stream_));
            }
        } else {
            SPH_CUDA(cudaMemsetAsync(bucket_, 0, sizeof(uint2) * total_buckets_, stream_));
        }
        SPH_CUDA(launch_keys_onesweep(pos_, tank_of_, d_tanks_, n, grid_.keys, passes, sweep_, stream_, compact_ids_));
        SPH_CUDA(launch_onesweep_sort(grid_, n, passes, sweep_, stream_, nullptr));
        SPH_CUDA(launch_bounds_gather(grid_.sorted_keys, grid_.sorted_ids, n, bucket_, pos_, vel_, tank_of_, spos_,
                                      svel_, stank_, schedule, stream_, compact_ids_, compact_sorted_));
        if ((status = enqueue_fields(nullptr)) != SPH_OK) {
            return status;
        }
        SPH_CUDA(launch_density(spos_, svel_, spos2_, bucket_, d_tanks_, stank_, n, nullptr, stream_, tuning));
        SPH_CUDA(launch_integrate(spos2_, svel_, compact_sorted_, bucket_, d_tanks_, stank_, n, pos_, vel_, stream_,
                                  tuning));
        if ((status = enqueue_colliders(nullptr)) != SPH_OK) {
            return status;
        }
    }
    return SPH_OK;
}

int Engine::run_per_tank(const std::vector<float>& dt, const std::vector<uint32_t>& substeps) {
    if (dt.size() != tanks_.size() || substeps.size() != tanks_.size()) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    uint32_t rounds = 0;
    for (size_t t = 0; t < tanks_.size(); ++t) {
        if (substeps[t] > 0 && (!(dt[t] > 0.0F) || !std::isfinite(dt[t]))) {
            return SPH_ERR_INVALID_ARGUMENT;
        }
        rounds = std::max(rounds, substeps[t]);
    }
    if (total_count_ == 0 || rounds == 0) {
        return SPH_OK;
    }
    SPH_CUDA(cudaSetDevice(device_));
    int status = ensure_graph();
    if (status != SPH_OK) {
        return status;
    }
    std::vector<uint32_t> chosen(tanks_.size());
    for (size_t t = 0; t < tanks_.size(); ++t) {
        chosen[t] = user_active_.empty() ? 1U : user_active_[t];
    }
    for (uint32_t r = 0; r < rounds; ++r) {
        // Tank t runs substeps[t] substeps of dt[t]; afterwards it sits out.
        for (size_t t = 0; t < tanks_.size(); ++t) {
            TankConst& k = tanks_[t];
            k.active = (r < substeps[t] && chosen[t] != 0) ? 1U : 0U;
            k.dt = dt[t];
            k.max_speed = dt[t] > 0.0F ? 0.4F * k.h / dt[t] : 0.0F;
        }
        SPH_CUDA(cudaMemcpyAsync(d_tanks_, tanks_.data(), tanks_.size() * sizeof(TankConst), cudaMemcpyHostToDevice,
                                 stream_));
        if ((status = prepare_schedule(nullptr)) != SPH_OK) {
            return status;
        }
        SPH_CUDA(cudaGraphLaunch(graph_, stream_));
    }
    for (size_t t = 0; t < tanks_.size(); ++t) {
        tanks_[t].active = chosen[t];
    }
    consts_dirty_ = true;
    grid_valid_ = true;
    return SPH_OK;
}

int Engine::stats_all(std::vector<sph_stats>& out) {
    out.assign(tanks_.size(), sph_stats{});
    SPH_CUDA(cudaSetDevice(device_));
    int status = refresh_constants(const_dt_ < 0.0F ? 0.0F : const_dt_);
    if (status != SPH_OK) {
        return status;
    }
    SPH_CUDA(cudaMemsetAsync(stats_acc_, 0, sizeof(double) * kStatsPerTank * tanks_.size(), stream_));
    SPH_CUDA(launch_stats(pos_, vel_, tank_of_, d_tanks_, total_count_, stats_acc_, stream_));
    std::vector<double> acc(kStatsPerTank * tanks_.size());
    SPH_CUDA(cudaMemcpyAsync(acc.data(), stats_acc_, sizeof(double) * acc.size(), cudaMemcpyDeviceToHost, stream_));
    SPH_CUDA(cudaStreamSynchronize(stream_));
    for (size_t t = 0; t < tanks_.size(); ++t) {
        const double* a = acc.data() + t * kStatsPerTank;
        sph_stats& o = out[t];
        o.particles = tanks_[t].particle_count;
        o.buckets = params_[t].lattice[3];
        double count = a[8];
        if (count > 0) {
            o.mean_density = a[0] / count;
            o.mean_compression = a[1] / count;
            o.centre_of_mass[0] = a[3] / count;
            o.centre_of_mass[1] = a[4] / count;
            o.centre_of_mass[2] = a[5] / count;
        }
        std::memcpy(&o.max_density, &a[2], sizeof(double));
        o.kinetic_energy = a[6];
        o.nonfinite = static_cast<uint32_t>(a[7]);
    }
    return SPH_OK;
}

int Engine::snapshot(bool save, uint32_t slot) {
    if (slot >= kSnapshotSlots) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    SPH_CUDA(cudaSetDevice(device_));
    if (snap_pos_[slot] == nullptr) {
        int status = SPH_OK;
        if ((status = alloc(&snap_pos_[slot], total_capacity_)) != SPH_OK ||
            (status = alloc(&snap_vel_[slot], total_capacity_)) != SPH_OK) {
            return status;
        }
    }
    size_t bytes = sizeof(float4) * total_count_;
    if (bytes == 0) {
        return SPH_OK;
    }
    if (save) {
        SPH_CUDA(cudaMemcpyAsync(snap_pos_[slot], pos_, bytes, cudaMemcpyDeviceToDevice, stream_));
        SPH_CUDA(cudaMemcpyAsync(snap_vel_[slot], vel_, bytes, cudaMemcpyDeviceToDevice, stream_));
    } else {
        SPH_CUDA(cudaMemcpyAsync(pos_, snap_pos_[slot], bytes, cudaMemcpyDeviceToDevice, stream_));
        SPH_CUDA(cudaMemcpyAsync(vel_, snap_vel_[slot], bytes, cudaMemcpyDeviceToDevice, stream_));
        grid_valid_ = false;
    }
    return SPH_OK;
}

int Engine::copy_state(float4* positions, float4* velocities) {
    SPH_CUDA(cudaSetDevice(device_));
    size_t bytes = sizeof(float4) * total_count_;
    if (positions != nullptr && bytes > 0) {
        SPH_CUDA(cudaMemcpyAsync(positions, pos_, bytes, cudaMemcpyDeviceToDevice, stream_));
    }
    if (velocities != nullptr && bytes > 0) {
        SPH_CUDA(cudaMemcpyAsync(velocities, vel_, bytes, cudaMemcpyDeviceToDevice, stream_));
    }
    return SPH_OK;
}

int Engine::restore_tanks(uint32_t slot, const std::vector<uint8_t>& which) {
    if (slot >= kSnapshotSlots || snap_pos_[slot] == nullptr || which.size() != tanks_.size()) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    SPH_CUDA(cudaSetDevice(device_));
    // Neighbouring selected tanks whose particles are adjacent share one copy.
    size_t first = 0;
    size_t count = 0;
    auto flush = [&]() -> int {
        if (count > 0) {
            size_t bytes = sizeof(float4) * count;
            SPH_CUDA(cudaMemcpyAsync(pos_ + first, snap_pos_[slot] + first, bytes, cudaMemcpyDeviceToDevice, stream_));
            SPH_CUDA(cudaMemcpyAsync(vel_ + first, snap_vel_[slot] + first, bytes, cudaMemcpyDeviceToDevice, stream_));
        }
        count = 0;
        return SPH_OK;
    };
    for (size_t t = 0; t < tanks_.size(); ++t) {
        if (which[t] == 0 || tanks_[t].particle_count == 0) {
            continue;
        }
        const size_t base = tanks_[t].particle_base;
        if (count > 0 && base != first + count) {
            int status = flush();
            if (status != SPH_OK) {
                return status;
            }
        }
        if (count == 0) {
            first = base;
        }
        count += tanks_[t].particle_count;
    }
    int status = flush();
    if (status != SPH_OK) {
        return status;
    }
    grid_valid_ = false;
    return SPH_OK;
}

int Engine::autotune(float dt, uint32_t substeps, TuneChoice* best, std::vector<TuneChoice>* tried) {
    if (best == nullptr || !(dt > 0.0F) || substeps == 0) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    if (total_count_ == 0) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    SPH_CUDA(cudaSetDevice(device_));
    cudaEvent_t start = nullptr;
    cudaEvent_t stop = nullptr;
    SPH_CUDA(cudaEventCreate(&start));
    SPH_CUDA(cudaEventCreate(&stop));
    int status = snapshot(true);
    const NeighbourTuning original = tuning_;
    const uint32_t original_bits = radix_bits_;
    const uint32_t original_schedule = schedule_curve_;
    const bool original_onesweep = onesweep_;
    const bool original_counting = counting_;
    auto measure = [&](const TuneChoice& c, float* ms) -> int {
        int st = set_tuning(c.tuning);
        if (st == SPH_OK) {
            st = set_schedule(c.schedule);
        }
        if (st == SPH_OK) {
            st = set_radix_bits(c.radix_bits);
        }
        if (st == SPH_OK) {
            st = set_onesweep(c.onesweep);
        }
        if (st == SPH_OK) {
            st = set_counting(c.counting);
        }
        if (st == SPH_OK) {
            st = snapshot(false);
        }
        if (st == SPH_OK) {
            st = run(dt, 1);  // captures the graph, warms caches
        }
        if (st != SPH_OK) {
            return st;
        }
        // At least one Morton order remake per timed run, so its cost counts.
        const uint32_t timed = std::max(substeps, kScheduleRefresh);
        SPH_CUDA(cudaEventRecord(start, stream_));
        st = run(dt, timed);
        if (st != SPH_OK) {
            return st;
        }
        SPH_CUDA(cudaEventRecord(stop, stream_));
        SPH_CUDA(cudaEventSynchronize(stop));
        SPH_CUDA(cudaEventElapsedTime(ms, start, stop));
        *ms /= static_cast<float>(timed);
        return SPH_OK;
    };
    // Stage 1: neighbour kernel, block size and processing order; stage 2:
    // the radix digit width for the winner.
    std::vector<TuneChoice> stage1;
    for (uint32_t variant : {3u, 4u}) {
        for (uint32_t block : {128u, 256u}) {
            for (uint32_t schedule : {0u, 1u, 2u}) {
                TuneChoice c;
                c.tuning = original;
                c.tuning.variant = variant;
                c.tuning.block = block;
                c.tuning.queue = 32;
                c.schedule = schedule;
                c.radix_bits = original_bits;
                c.onesweep = original_onesweep;
                c.counting = original_counting;
                stage1.push_back(c);
            }
        }
    }
    TuneChoice winner;
    winner.ms = 1e30F;
    for (TuneChoice& c : stage1) {
        if (status == SPH_OK) {
            status = measure(c, &c.ms);
        }
        if (status == SPH_OK && c.ms < winner.ms) {
            winner = c;
        }
        if (tried != nullptr) {
            tried->push_back(c);
        }
    }
    // Stage 2: the grid sort (counting placement, one-sweep, or three kernels
    // per pass at 5-8 bits).
    const TuneChoice stage1_winner = winner;
    for (uint32_t bits : {1u, 0u, 5u, 6u, 7u, 8u}) {
        TuneChoice c = stage1_winner;
        c.counting = bits == 1;
        c.onesweep = bits <= 1;
        c.radix_bits = bits <= 1 ? stage1_winner.radix_bits : bits;
        if (status != SPH_OK ||
            (c.counting == stage1_winner.counting && c.onesweep == stage1_winner.onesweep &&
             (c.counting || c.onesweep || c.radix_bits == stage1_winner.radix_bits))) {
            continue;
        }
        status = measure(c, &c.ms);
        if (status == SPH_OK && c.ms < winner.ms) {
            winner = c;
        }
        if (tried != nullptr) {
            tried->push_back(c);
        }
    }
    int restore = snapshot(false);
    if (status == SPH_OK) {
        status = restore;
    }
    if (status == SPH_OK) {
        status = set_tuning(winner.tuning);
        if (status == SPH_OK) {
            status = set_schedule(winner.schedule);
        }
        if (status == SPH_OK) {
            status = set_radix_bits(winner.radix_bits);
        }
        if (status == SPH_OK) {
            status = set_onesweep(winner.onesweep);
        }
        if (status == SPH_OK) {
            status = set_counting(winner.counting);
        }
        *best = winner;
    } else {
        set_tuning(original);
        set_schedule(original_schedule);
        set_radix_bits(original_bits);
        set_onesweep(original_onesweep);
        set_counting(original_counting);
    }
    cudaEventDestroy(start);
    cudaEventDestroy(stop);
    return status;
}

int Engine::ensure_learned_buffers() {
    if (sforce_ != nullptr) {
        return SPH_OK;
    }
    int status = SPH_OK;
    if ((status = alloc(&sforce_, total_capacity_)) != SPH_OK ||
        (status = alloc(&scorrection_, total_capacity_)) != SPH_OK ||
        (status = alloc(&correction_sums_, tanks_.size() * kCorrectionSumWords)) != SPH_OK ||
        (status = alloc(&sfeatures_, static_cast<size_t>(total_capacity_) * 32)) != SPH_OK ||
        (status = alloc(&sx_tiles_, static_cast<size_t>((total_capacity_ + mlp::kTile - 1) / mlp::kTile) *
                                        mlp::kXTileBytes)) != SPH_OK) {
        return status;
    }
    SPH_CUDA(mlp::prepare_forward());
    return SPH_OK;
}

// One learned substep: grid, density (with the pair masks), force +
// features, MLP, finish. model == nullptr runs the same split path with a
// zero correction (bit-identical to the plain substep).
int Engine::enqueue_learned_substep(const mlp::ModelView* model, uint32_t* launches) {
    int status = enqueue_grid(launches);
    if (status != SPH_OK) {
        return status;
    }
    uint32_t n = total_count_;
    NeighbourTuning masked = tuning_;
    masked.variant = 4;
    if ((status = enqueue_fields(launches)) != SPH_OK) {
        return status;
    }
    const bool free = model != nullptr && model->free_axes != 0;
    SPH_CUDA(launch_density(spos_, svel_, spos2_, bucket_, d_tanks_, stank_, n, nullptr, stream_, masked));
    if (free) {  // zeroed here, so that nothing but kernels sits between features and finish
        SPH_CUDA(zero_correction_sums(static_cast<uint32_t>(tanks_.size()), correction_sums_, stream_));
    }
    // The features go straight into the MLP's input tiles (normalised, BF16);
    // with no model only the plain force is needed. The MLP, the sums and
    // the finishing pass are programmatic dependents, each waiting for the
    // grid before it: their set-up overlaps that grid's last blocks.
    SPH_CUDA(launch_features(spos2_, svel_, grid_.sorted_ids, bucket_, d_tanks_, stank_, n, tuning_.order,
                             tuning_.masks, sforce_, nullptr, false, stream_,
                             model != nullptr ? model->in_mean : nullptr, model != nullptr ? model->in_inv_std : nullptr,
                             model != nullptr ? sx_tiles_ : nullptr));
    if (model != nullptr) {
        SPH_CUDA(mlp::launch_forward_tiles(*model, sx_tiles_, n, reinterpret_cast<float*>(scorrection_),
                                           &counters_->error_flags, stream_, true));
        if (free) {
            // No net force along these axes: each tank's mean correction is removed.
            SPH_CUDA(launch_correction_sums(scorrection_, d_tanks_, stank_, n, static_cast<uint32_t>(tanks_.size()),
                                            correction_sums_, stream_, true));
        }
    }
    SPH_CUDA(launch_finish_learned(spos2_, svel_, grid_.sorted_ids, d_tanks_, stank_, n, sforce_,
                                   model != nullptr ? scorrection_ : nullptr, free ? correction_sums_ : nullptr,
                                   free ? model->free_axes : 0u, pos_, vel_, stream_, true));
    if (launches != nullptr) {
        *launches += model != nullptr ? (free ? 5 : 4) : 3;
    }
    return enqueue_colliders(launches);
}

int Engine::run_learned(float dt, uint32_t substeps, const mlp::ModelView* model) {
    if (!(dt > 0.0F) || !std::isfinite(dt)) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    if (total_count_ == 0 || substeps == 0) {
        return SPH_OK;
    }
    SPH_CUDA(cudaSetDevice(device_));
    int status = ensure_learned_buffers();
    if (status != SPH_OK) {
        return status;
    }
    status = refresh_constants(dt);
    if (status != SPH_OK) {
        return status;
    }
    bool same_model = (model == nullptr && !learned_graph_has_model_) ||
                      (model != nullptr && learned_graph_has_model_ &&
                       std::memcmp(model, &learned_graph_model_, sizeof(mlp::ModelView)) == 0);
    if (learned_graph_ == nullptr || learned_graph_count_ != total_count_ || !same_model) {
        if (learned_graph_ != nullptr) {
            cudaGraphExecDestroy(learned_graph_);
            learned_graph_ = nullptr;
        }
        SPH_CUDA(cudaMemsetAsync(&counters_->error_flags, 0, sizeof(unsigned int), stream_));
        if ((status = prepare_schedule(nullptr)) != SPH_OK) {
            return status;
        }
        cudaGraph_t graph = nullptr;
        SPH_CUDA(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
        uint32_t launches = 0;
        capturing_ = true;
        status = enqueue_learned_substep(model, &launches);
        capturing_ = false;
        cudaError_t end = cudaStreamEndCapture(stream_, &graph);
        if (status != SPH_OK) {
            if (graph != nullptr) {
                cudaGraphDestroy(graph);
            }
            return status;
        }
        if (end != cudaSuccess) {
            return fail(end, "cudaStreamEndCapture");
        }
        cudaError_t inst = cudaGraphInstantiate(&learned_graph_, graph, 0);
        cudaGraphDestroy(graph);
        if (inst != cudaSuccess) {
            learned_graph_ = nullptr;
            return fail(inst, "cudaGraphInstantiate");
        }
        learned_graph_count_ = total_count_;
        learned_graph_has_model_ = model != nullptr;
        if (model != nullptr) {
            learned_graph_model_ = *model;
        }
        learned_launches_ = launches;
    }
    for (uint32_t s = 0; s < substeps; ++s) {
        if ((status = prepare_schedule(nullptr)) != SPH_OK) {
            return status;
        }
        SPH_CUDA(cudaGraphLaunch(learned_graph_, stream_));
    }
    grid_valid_ = true;
    return SPH_OK;
}

int Engine::learned_error() {
    unsigned int flag = 0;
    SPH_CUDA(cudaMemcpyAsync(&flag, &counters_->error_flags, sizeof(flag), cudaMemcpyDeviceToHost, stream_));
    SPH_CUDA(cudaStreamSynchronize(stream_));
    if (flag != 0) {
        last_error_ = "tensor-core completion wait timed out";
        return SPH_ERR_TIMEOUT;
    }
    return SPH_OK;
}

// Features of the current state (id order), for training sets; the state
// itself does not change.
int Engine::learned_features(float dt, float* features) {
    if (features == nullptr || !(dt > 0.0F)) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    if (total_count_ == 0) {
        return SPH_OK;
    }
    SPH_CUDA(cudaSetDevice(device_));
    int status = ensure_learned_buffers();
    if (status == SPH_OK) {
        status = refresh_constants(dt);
    }
    if (status == SPH_OK) {
        status = enqueue_grid(nullptr);
    }
    if (status != SPH_OK) {
        return status;
    }
    uint32_t n = total_count_;
    NeighbourTuning masked = tuning_;
    masked.variant = 4;
    masked.all_tanks = true;  // features of every tank, active or not
    SPH_CUDA(launch_density(spos_, svel_, spos2_, bucket_, d_tanks_, stank_, n, nullptr, stream_, masked));
    SPH_CUDA(launch_features(spos2_, svel_, grid_.sorted_ids, bucket_, d_tanks_, stank_, n, tuning_.order,
                             tuning_.masks, sforce_, features, true, stream_));
    grid_valid_ = true;
    return SPH_OK;
}

// The correction of a learned substep from the current state, through the
// learned step's own kernels (BF16 input tiles, the tiled forward pass), in
// id order; the state does not change.
int Engine::learned_correction(float dt, const mlp::ModelView& model, float4* correction) {
    if (correction == nullptr || !(dt > 0.0F)) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    if (total_count_ == 0) {
        return SPH_OK;
    }
    SPH_CUDA(cudaSetDevice(device_));
    int status = ensure_learned_buffers();
    if (status == SPH_OK) {
        status = refresh_constants(dt);
    }
    if (status == SPH_OK) {
        status = enqueue_grid(nullptr);
    }
    if (status != SPH_OK) {
        return status;
    }
    uint32_t n = total_count_;
    NeighbourTuning masked = tuning_;
    masked.variant = 4;
    SPH_CUDA(mlp::prepare_forward());
    SPH_CUDA(launch_density(spos_, svel_, spos2_, bucket_, d_tanks_, stank_, n, nullptr, stream_, masked));
    SPH_CUDA(launch_features(spos2_, svel_, grid_.sorted_ids, bucket_, d_tanks_, stank_, n, tuning_.order,
                             tuning_.masks, sforce_, nullptr, false, stream_, model.in_mean, model.in_inv_std,
                             sx_tiles_));
    SPH_CUDA(mlp::launch_forward_tiles(model, sx_tiles_, n, reinterpret_cast<float*>(scorrection_),
                                       &counters_->error_flags, stream_));
    SPH_CUDA(launch_scatter_rows(scorrection_, grid_.sorted_ids, n, correction, stream_));
    grid_valid_ = true;
    return learned_error();
}

int Engine::build_grid() {
    SPH_CUDA(cudaSetDevice(device_));
    int status = refresh_constants(const_dt_ < 0.0F ? 0.0F : const_dt_);
    if (status != SPH_OK) {
        return status;
    }
    status = enqueue_grid(nullptr);
    if (status == SPH_OK) {
        grid_valid_ = true;
    }
    return status;
}

int Engine::grid_download(uint32_t tank, uint32_t* cell_of, uint32_t* cell_counts, uint32_t* cell_particles) {
    if (tank >= tanks_.size()) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    if (!grid_valid_) {
        int status = build_grid();
        if (status != SPH_OK) {
            return status;
        }
    }
    SPH_CUDA(cudaSetDevice(device_));
    SPH_CUDA(cudaStreamSynchronize(stream_));
    // The sort buffers an earlier substep left hold its result.
    if (grid_.sorted_ids == nullptr) {
        RadixPlan p = plan_;
        grid_.sorted_keys = p.passes % 2 == 1 ? grid_.keys_a : grid_.keys_b;
        grid_.sorted_ids = p.passes % 2 == 1 ? grid_.vals_a : grid_.vals_b;
    }
    const TankConst& t = tanks_[tank];
    uint32_t n = t.particle_count;
    uint32_t cells = params_[tank].lattice[3];
    if (cell_of != nullptr && n > 0) {
        SPH_CUDA(cudaMemcpy(cell_of, grid_.keys + t.particle_base, n * sizeof(uint32_t), cudaMemcpyDeviceToHost));
        for (uint32_t i = 0; i < n; ++i) {
            cell_of[i] -= t.bucket_base;
        }
    }
    std::vector<uint2> table(cells);
    SPH_CUDA(cudaMemcpy(table.data(), bucket_ + t.bucket_base, cells * sizeof(uint2), cudaMemcpyDeviceToHost));
    if (cell_counts != nullptr) {
        for (uint32_t b = 0; b < cells; ++b) {
            cell_counts[b] = table[b].y - table[b].x;
        }
    }
    if (cell_particles != nullptr && total_count_ > 0) {
        std::vector<uint32_t> ids(total_count_);
        SPH_CUDA(cudaMemcpy(ids.data(), grid_.sorted_ids, total_count_ * sizeof(uint32_t), cudaMemcpyDeviceToHost));
        for (uint32_t b = 0; b < cells; ++b) {
            uint32_t count = std::min(table[b].y - table[b].x, kCellCapacity);
            for (uint32_t k = 0; k < count; ++k) {
                cell_particles[static_cast<size_t>(b) * kCellCapacity + k] = ids[table[b].x + k] - t.particle_base;
            }
        }
    }
    return SPH_OK;
}

int Engine::stats(uint32_t tank, sph_stats* out, bool with_pairs) {
    if (tank >= tanks_.size() || out == nullptr) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    std::memset(out, 0, sizeof(*out));
    SPH_CUDA(cudaSetDevice(device_));
    int status = refresh_constants(const_dt_ < 0.0F ? 0.0F : const_dt_);
    if (status != SPH_OK) {
        return status;
    }
    uint32_t n = total_count_;
    SPH_CUDA(cudaMemsetAsync(stats_acc_, 0, sizeof(double) * kStatsPerTank * tanks_.size(), stream_));
    SPH_CUDA(launch_stats(pos_, vel_, tank_of_, d_tanks_, n, stats_acc_, stream_));
    StepCounters counters{};
    uint32_t bucket_info[2] = {0, 0};
    if (with_pairs && n > 0) {
        status = enqueue_grid(nullptr);
        if (status != SPH_OK) {
            return status;
        }
        grid_valid_ = true;
        SPH_CUDA(cudaMemsetAsync(counters_, 0, sizeof(StepCounters), stream_));
        SPH_CUDA(launch_density(spos_, svel_, spos2_, bucket_, d_tanks_, stank_, n, counters_, stream_, tuning_));
        SPH_CUDA(cudaMemsetAsync(bucket_stats_, 0, 2 * sizeof(uint32_t), stream_));
        SPH_CUDA(launch_bucket_stats(bucket_ + tanks_[tank].bucket_base, params_[tank].lattice[3], bucket_stats_,
                                     stream_));
        SPH_CUDA(cudaMemcpyAsync(&counters, counters_, sizeof(StepCounters), cudaMemcpyDeviceToHost, stream_));
        SPH_CUDA(cudaMemcpyAsync(bucket_info, bucket_stats_, sizeof(bucket_info), cudaMemcpyDeviceToHost, stream_));
    }
    std::vector<double> acc(kStatsPerTank * tanks_.size());
    SPH_CUDA(cudaMemcpyAsync(acc.data(), stats_acc_, sizeof(double) * acc.size(), cudaMemcpyDeviceToHost, stream_));
    SPH_CUDA(cudaStreamSynchronize(stream_));
    const double* a = acc.data() + static_cast<size_t>(tank) * kStatsPerTank;
    double count = a[8];
    out->particles = tanks_[tank].particle_count;
    out->buckets = params_[tank].lattice[3];
    out->max_bucket_count = bucket_info[0];
    out->overflow_buckets = bucket_info[1];
    out->candidates = tanks_.size() == 1 ? counters.candidates : 0;
    out->pairs_in_range = tanks_.size() == 1 ? counters.in_range : 0;
    if (count > 0) {
        out->mean_density = a[0] / count;
        out->mean_compression = a[1] / count;
        out->centre_of_mass[0] = a[3] / count;
        out->centre_of_mass[1] = a[4] / count;
        out->centre_of_mass[2] = a[5] / count;
    }
    uint64_t bits = 0;
    std::memcpy(&bits, &a[2], sizeof(bits));
    std::memcpy(&out->max_density, &bits, sizeof(bits));
    out->kinetic_energy = a[6];
    out->nonfinite = static_cast<uint32_t>(a[7]);
    return SPH_OK;
}

int Engine::synchronize() {
    SPH_CUDA(cudaSetDevice(device_));
    SPH_CUDA(cudaStreamSynchronize(stream_));
    return SPH_OK;
}

int Engine::set_active(const std::vector<uint8_t>& active) {
    if (active.size() != tanks_.size()) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    user_active_ = active;
    for (size_t t = 0; t < tanks_.size(); ++t) {
        tanks_[t].active = active[t] != 0 ? 1U : 0U;
    }
    active_dirty_ = true;  // only the flags go up (refresh_constants)
    return SPH_OK;
}

int Engine::selftest_division(uint64_t seed, uint64_t count, int mode, uint64_t* mismatches) {
    if (mismatches == nullptr || mode < 0 || mode > 6) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    SPH_CUDA(cudaSetDevice(device_));
    SPH_CUDA(cudaMemsetAsync(counters_, 0, sizeof(StepCounters), stream_));
    SPH_CUDA(launch_division_selftest(seed, count, mode, &counters_->candidates, stream_));
    unsigned long long bad = 0;
    SPH_CUDA(cudaMemcpyAsync(&bad, &counters_->candidates, sizeof(bad), cudaMemcpyDeviceToHost, stream_));
    SPH_CUDA(cudaStreamSynchronize(stream_));
    *mismatches = bad;
    return SPH_OK;
}

int Engine::set_tuning(const NeighbourTuning& tuning) {
    bool queue_ok = tuning.queue == 8 || tuning.queue == 16 || tuning.queue == 24 || tuning.queue == 32;
    if (tuning.variant > 6 || tuning.block < 32 || tuning.block > 512 || tuning.block % 32 != 0 || !queue_ok ||
        static_cast<size_t>(tuning.queue) * tuning.block * sizeof(uint32_t) > 48 * 1024) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    if (tuning.variant >= 2 && tuning.block != 64 && tuning.block != 128 && tuning.block != 256) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    if (tuning.variant == 6 && tuning.block != 128 && tuning.block != 256) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    NeighbourTuning kept = tuning_;
    tuning_ = tuning;
    tuning_.pair_list = kept.pair_list;
    tuning_.pair_count = kept.pair_count;
    tuning_.list_cap = kept.list_cap;
    tuning_.masks = kept.masks;
    tuning_.order = kept.order;
    if (graph_ != nullptr) {
        cudaGraphExecDestroy(graph_);
        graph_ = nullptr;
    }
    drop_host_graph();
    return SPH_OK;
}

int Engine::set_counting(bool on) {
    counting_ = on;
    return set_onesweep(onesweep_);  // drops the graphs and the grid as a sort change does
}

int Engine::set_onesweep(bool on) {
    onesweep_ = on;
    if (graph_ != nullptr) {
        cudaGraphExecDestroy(graph_);
        graph_ = nullptr;
    }
    drop_host_graph();
    if (learned_graph_ != nullptr) {
        cudaGraphExecDestroy(learned_graph_);
        learned_graph_ = nullptr;
    }
    grid_.sorted_keys = nullptr;
    grid_.sorted_ids = nullptr;
    grid_valid_ = false;
    return SPH_OK;
}

int Engine::set_schedule(uint32_t curve) {
    if (curve > 2) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    schedule_curve_ = curve;
    rank_count_ = 0xFFFFFFFFu;
    if (graph_ != nullptr) {
        cudaGraphExecDestroy(graph_);
        graph_ = nullptr;
    }
    drop_host_graph();
    grid_valid_ = false;
    return SPH_OK;
}

int Engine::set_radix_bits(uint32_t bits) {
    if (bits < 1 || bits > kRadixMaxBits) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    radix_bits_ = bits;
    plan_ = plan_radix(bit_width(total_buckets_ - 1U), radix_bits_);
    if (graph_ != nullptr) {
        cudaGraphExecDestroy(graph_);
        graph_ = nullptr;
    }
    drop_host_graph();
    grid_.sorted_keys = nullptr;
    grid_.sorted_ids = nullptr;
    grid_valid_ = false;
    return SPH_OK;
}

int Engine::profile(float dt, uint32_t substeps, double* phase_ms) {
    if (phase_ms == nullptr || !(dt > 0.0F)) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    for (uint32_t k = 0; k < kProfilePhases; ++k) {
        phase_ms[k] = 0.0;
    }
    if (total_count_ == 0) {
        return SPH_OK;
    }
    SPH_CUDA(cudaSetDevice(device_));
    int status = refresh_constants(dt);
    if (status != SPH_OK) {
        return status;
    }
    if (events_[0] == nullptr) {
        for (cudaEvent_t& e : events_) {
            SPH_CUDA(cudaEventCreate(&e));
        }
    }
    uint32_t n = total_count_;
    for (uint32_t s = 0; s < substeps; ++s) {
        SPH_CUDA(cudaEventRecord(events_[0], stream_));
        if ((status = prepare_schedule(nullptr)) != SPH_OK) {  // counted with the keys
            return status;
        }
        const uint32_t passes = onesweep_passes(bit_width(total_buckets_ - 1U));
        if (counting_) {
            // keys: the whole counting placement; sort: nothing left.
            SPH_CUDA(launch_counting_grid(pos_, tank_of_, d_tanks_, n, total_buckets_, grid_, counts_, block_sums_,
                                          bucket_, stream_, nullptr));
        } else if (onesweep_) {
            SPH_CUDA(cudaMemsetAsync(bucket_, 0, sizeof(uint2) * total_buckets_, stream_));
            SPH_CUDA(launch_keys_onesweep(pos_, tank_of_, d_tanks_, n, grid_.keys, passes, sweep_, stream_));
        } else {
            SPH_CUDA(cudaMemsetAsync(bucket_, 0, sizeof(uint2) * total_buckets_, stream_));
            SPH_CUDA(launch_keys(pos_, tank_of_, d_tanks_, n, grid_.keys, stream_));
        }
        SPH_CUDA(cudaEventRecord(events_[1], stream_));
        if (!counting_ && onesweep_) {
            SPH_CUDA(launch_onesweep_sort(grid_, n, passes, sweep_, stream_, nullptr));
        } else if (!counting_) {
            SPH_CUDA(launch_radix_sort(grid_, n, plan_, stream_, nullptr));
        }
        SPH_CUDA(cudaEventRecord(events_[2], stream_));
        status = enqueue_bounds(nullptr);
        if (status != SPH_OK) {
            return status;
        }
        SPH_CUDA(cudaEventRecord(events_[3], stream_));
        SPH_CUDA(launch_density(spos_, svel_, spos2_, bucket_, d_tanks_, stank_, n, nullptr, stream_, tuning_));
        SPH_CUDA(cudaEventRecord(events_[4], stream_));
        // Force fields (before integrate, at the start positions) and
        // colliders (after it), when present, make up the shapes phase.
        if ((status = enqueue_fields(nullptr)) != SPH_OK) {
            return status;
        }
        SPH_CUDA(cudaEventRecord(events_[5], stream_));
        SPH_CUDA(launch_integrate(spos2_, svel_, grid_.sorted_ids, bucket_, d_tanks_, stank_, n, pos_, vel_, stream_,
                                  tuning_));
        SPH_CUDA(cudaEventRecord(events_[6], stream_));
        if ((status = enqueue_colliders(nullptr)) != SPH_OK) {
            return status;
        }
        SPH_CUDA(cudaEventRecord(events_[7], stream_));
        SPH_CUDA(cudaEventSynchronize(events_[7]));
        float ms[7] = {};
        for (uint32_t k = 0; k < 7; ++k) {
            SPH_CUDA(cudaEventElapsedTime(&ms[k], events_[k], events_[k + 1]));
        }
        // keys, sort, bounds + gather, density, integrate, shapes.
        const float phase[kProfilePhases] = {ms[0], ms[1], ms[2], ms[3], ms[5], ms[4] + ms[6]};
        for (uint32_t k = 0; k < kProfilePhases; ++k) {
            phase_ms[k] += phase[k];
        }
    }
    grid_valid_ = true;
    return SPH_OK;
}

// ---- fluid surface ----------------------------------------------------------------

int Engine::grow(void** buffer, size_t* have, size_t need) {
    if (*buffer != nullptr && *have >= need) {
        return SPH_OK;
    }
    if (*buffer != nullptr) {
        SPH_CUDA(cudaStreamSynchronize(stream_));
        SPH_CUDA(cudaFree(*buffer));
        device_bytes_ -= *have;
        *buffer = nullptr;
        *have = 0;
    }
    SPH_CUDA(cudaMalloc(buffer, std::max<size_t>(need, 16)));
    *have = std::max<size_t>(need, 16);
    device_bytes_ += *have;
    return SPH_OK;
}

int Engine::surface_field(uint32_t tank, uint32_t resolution) {
    if (tank >= tanks_.size() || resolution == 0 || resolution > SPH_SURFACE_MAX_RESOLUTION) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    SPH_CUDA(cudaSetDevice(device_));
    const uint64_t samples = resolution + 1ull;
    int status = grow(reinterpret_cast<void**>(&surface_field_), &surface_field_bytes_,
                      samples * samples * samples * sizeof(float));
    if (status == SPH_OK) {
        status = grow(&surface_runs_, &surface_runs_bytes_, sizeof(surface::FieldRuns));
    }
    if (status != SPH_OK) {
        return status;
    }
    const sph_params& p = params_[tank];
    surface::FieldGeom g{};
    for (int a = 0; a < 3; ++a) {
        // buildFluidField (marching_cubes.cpp:375-378): cell = (max - min) / resolution.
        g.origin[a] = p.container_min[a];
        g.cell[a] = (p.container_max[a] - p.container_min[a]) / static_cast<float>(resolution);
    }
    g.radius = p.smoothing_radius;
    g.radius_sq = g.radius * g.radius;
    g.mask = p.lattice[3] - 1U;
    g.resolution = resolution;
    surface_resolution_ = resolution;
    surface_tank_ = tank;
    surface_written_ = 0;
    if (tanks_[tank].particle_count == 0 || total_count_ == 0) {
        SPH_CUDA(cudaMemsetAsync(surface_field_, 0, samples * samples * samples * sizeof(float), stream_));
        return SPH_OK;
    }
    // The grid of the current positions (the solver's own grid is from
    // before the last integration, marching_cubes.cpp:370-371).
    status = build_grid();
    if (status != SPH_OK) {
        return status;
    }
    SPH_CUDA(surface::launch_field(spos_, bucket_ + tanks_[tank].bucket_base, g,
                                   static_cast<surface::FieldRuns*>(surface_runs_), surface_field_, stream_));
    return SPH_OK;
}

int Engine::surface_march(float iso, uint32_t capacity, uint32_t* written) {
    if (written == nullptr || surface_resolution_ == 0) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    *written = 0;
    surface_written_ = 0;
    if (capacity < 3) {
        return SPH_OK;
    }
    SPH_CUDA(cudaSetDevice(device_));
    const uint32_t r = surface_resolution_;
    const uint32_t tiles = surface::march_tiles(r);
    int status = grow(reinterpret_cast<void**>(&surface_vertices_), &surface_vertices_bytes_,
                      static_cast<size_t>(capacity) * sizeof(sph_surface_vertex));
    if (status == SPH_OK) {
        status = grow(reinterpret_cast<void**>(&surface_codes_), &surface_codes_bytes_,
                      static_cast<size_t>(r) * r * r);
    }
    if (status == SPH_OK) {
        status = grow(reinterpret_cast<void**>(&surface_tiles_), &surface_tiles_bytes_,
                      (2 * static_cast<size_t>(tiles) + 2) * sizeof(uint32_t));
    }
    if (status != SPH_OK) {
        return status;
    }
    const sph_params& p = params_[surface_tank_];
    surface::MarchGeom g{};
    for (int a = 0; a < 3; ++a) {
        g.origin[a] = p.container_min[a];
        g.cell[a] = (p.container_max[a] - p.container_min[a]) / static_cast<float>(r);
    }
    g.iso = iso;
    g.resolution = r;
    surface::MarchScratch scratch{surface_codes_, surface_tiles_, surface_tiles_ + tiles,
                                  surface_tiles_ + 2 * static_cast<size_t>(tiles) + 1};
    SPH_CUDA(surface::launch_march(surface_field_, g, capacity, scratch, surface_vertices_, stream_));
    uint32_t total_and_limit[2] = {0, 0};
    SPH_CUDA(cudaMemcpyAsync(&total_and_limit[0], scratch.offsets + tiles, sizeof(uint32_t), cudaMemcpyDeviceToHost,
                             stream_));
    SPH_CUDA(cudaMemcpyAsync(&total_and_limit[1], scratch.limit, sizeof(uint32_t), cudaMemcpyDeviceToHost, stream_));
    SPH_CUDA(cudaStreamSynchronize(stream_));
    surface_written_ = std::min(total_and_limit[0], total_and_limit[1]);
    *written = surface_written_;
    return SPH_OK;
}

int Engine::surface_field_download(float* out) {
    if (out == nullptr || surface_resolution_ == 0) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    SPH_CUDA(cudaSetDevice(device_));
    const size_t samples = surface_resolution_ + 1ull;
    SPH_CUDA(cudaMemcpyAsync(out, surface_field_, samples * samples * samples * sizeof(float), cudaMemcpyDeviceToHost,
                             stream_));
    SPH_CUDA(cudaStreamSynchronize(stream_));
    return SPH_OK;
}

int Engine::surface_vertices_download(sph_surface_vertex* out, uint32_t count) {
    if ((out == nullptr && count > 0) || count > surface_written_) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    if (count == 0) {
        return SPH_OK;
    }
    SPH_CUDA(cudaSetDevice(device_));
    SPH_CUDA(cudaMemcpyAsync(out, surface_vertices_, static_cast<size_t>(count) * sizeof(sph_surface_vertex),
                             cudaMemcpyDeviceToHost, stream_));
    SPH_CUDA(cudaStreamSynchronize(stream_));
    return SPH_OK;
}

}  // namespace sph
