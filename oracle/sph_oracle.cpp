// sph_oracle.cpp — CPU oracle of the reference's SPH fluid step.
//
// TEST INFRASTRUCTURE ONLY: the checker for the CUDA path and the timed CPU
// baseline. Every function names the reference lines it restates. Built with
// -ffp-contract=off -fno-fast-math so that each float operation is rounded
// once, in the order the reference writes it (GCC on aarch64 would otherwise
// fuse a*b+c into one FMA).
#include "sph_oracle.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

namespace {

// std::numbers::pi_v<float> (fluid_sph.cpp:20).
constexpr float PI = 3.14159265358979323846F;
// fluid_sph.cpp:22: chunk size of every parallel loop.
constexpr uint32_t GRANULARITY = 256;
constexpr uint32_t CAPACITY = SPH_CELL_CAPACITY;

struct V3 {
    float x, y, z;
};

inline V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 add(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 scale(float s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline V3 divide(V3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
// glm::dot for vec3: (x*x' + y*y') + z*z'.
inline float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
// glm::length: sqrt(dot(v, v)).
inline float length(V3 a) { return std::sqrt(dot(a, a)); }
inline V3 xyz(const float* v4) { return {v4[0], v4[1], v4[2]}; }

struct Cell {
    int32_t x, y, z;
};

// spatial_hash.h:12-14: ivec3(floor(p / h)), division per component.
inline Cell spatialCell(V3 p, float h) {
    return {static_cast<int32_t>(std::floor(p.x / h)), static_cast<int32_t>(std::floor(p.y / h)),
            static_cast<int32_t>(std::floor(p.z / h))};
}

// spatial_hash.h:16-20.
inline uint32_t spatialHash(Cell c, uint32_t cellCount) {
    uint32_t hashed = static_cast<uint32_t>(c.x) * 73856093U ^ static_cast<uint32_t>(c.y) * 19349663U ^
                      static_cast<uint32_t>(c.z) * 83492791U;
    return hashed & (cellCount - 1U);
}

// fluid_sph.cpp:24-31.
inline float poly6(float squaredDistance, float h) {
    float h2 = h * h;
    if (squaredDistance >= h2) {
        return 0.0F;
    }
    float d = h2 - squaredDistance;
    return 315.0F / (64.0F * PI * std::pow(h, 9.0F)) * d * d * d;
}

// fluid_sph.cpp:33-39.
inline V3 spikyGradient(V3 delta, float len, float h) {
    if (len >= h || len <= 1e-6F) {
        return {0.0F, 0.0F, 0.0F};
    }
    float d = h - len;
    return scale(-45.0F / (PI * std::pow(h, 6.0F)) * d * d, divide(delta, len));
}

// fluid_sph.cpp:41-46.
inline float viscosityLaplacian(float len, float h) {
    if (len >= h) {
        return 0.0F;
    }
    return 45.0F / (PI * std::pow(h, 6.0F)) * (h - len);
}

// force_field.h:31-60.
V3 forceFieldAcceleration(const sph_force_field& field, V3 position) {
    V3 offset = sub(position, {field.position_radius[0], field.position_radius[1], field.position_radius[2]});
    float distance = length(offset);
    float weight = 1.0F;
    float radius = field.position_radius[3];
    if (radius > 0.0F) {
        float t = std::clamp(1.0F - distance / radius, 0.0F, 1.0F);
        weight = t <= 0.0F ? 0.0F : std::pow(t, field.falloff);
    }
    if (weight <= 0.0F) {
        return {0.0F, 0.0F, 0.0F};
    }
    V3 axis{field.axis_strength[0], field.axis_strength[1], field.axis_strength[2]};
    float strength = field.axis_strength[3];
    switch (field.type) {
    case 0:
        return scale(strength * weight, axis);
    case 1: {
        V3 radial = sub(offset, scale(dot(offset, axis), axis));
        float r = length(radial);
        if (r < 1.0e-4F) {
            return {0.0F, 0.0F, 0.0F};
        }
        V3 u = divide(radial, r);
        V3 c{axis.y * u.z - u.y * axis.z, axis.z * u.x - u.z * axis.x, axis.x * u.y - u.x * axis.y};
        return scale(strength * weight, c);
    }
    case 2:
        if (distance < 1.0e-4F) {
            return {0.0F, 0.0F, 0.0F};
        }
        return scale(strength * weight, divide({-offset.x, -offset.y, -offset.z}, distance));
    default:
        return {0.0F, 0.0F, 0.0F};
    }
}

// force_field.h:62-70: starts from vec3{0} and adds every field.
V3 forceFieldsAcceleration(const sph_params& params, V3 position) {
    V3 total{0.0F, 0.0F, 0.0F};
    for (uint32_t i = 0; i < params.field_count && i < SPH_MAX_FORCE_FIELDS; ++i) {
        total = add(total, forceFieldAcceleration(params.fields[i], position));
    }
    return total;
}

// ---- shape colliders (collider_shapes.h:27-137, fluid_sph.cpp:48-53, :287-300)

struct Surface {
    V3 point{0.0F, 0.0F, 0.0F};
    V3 normal{0.0F, 1.0F, 0.0F};
    float distance = 0.0F;
};

inline float clampf(float v, float lo, float hi) { return v < lo ? lo : (hi < v ? hi : v); }  // std::clamp
inline float minf(float a, float b) { return b < a ? b : a; }                                  // std::min
inline float maxf(float a, float b) { return a < b ? b : a; }                                  // std::max

// collider_shapes.h:33-41.
Surface closestOnSphere(float radius, V3 p) {
    Surface r;
    float d = length(p);
    r.normal = d > 1.0e-6F ? divide(p, d) : V3{0.0F, 1.0F, 0.0F};
    r.point = scale(radius, r.normal);
    r.distance = d - radius;
    return r;
}

// collider_shapes.h:44-66; glm::clamp is min(max(v, lo), hi) per component.
Surface closestOnBox(V3 extent, V3 p) {
    Surface r;
    V3 clamped{minf(maxf(p.x, -extent.x), extent.x), minf(maxf(p.y, -extent.y), extent.y),
               minf(maxf(p.z, -extent.z), extent.z)};
    V3 delta = sub(p, clamped);
    float distanceSq = dot(delta, delta);
    if (distanceSq > 1.0e-10F) {
        float distance = std::sqrt(distanceSq);
        r.normal = divide(delta, distance);
        r.point = clamped;
        r.distance = distance;
        return r;
    }
    float gap[3] = {extent.x - std::fabs(p.x), extent.y - std::fabs(p.y), extent.z - std::fabs(p.z)};
    int axis = gap[0] < gap[1] ? (gap[0] < gap[2] ? 0 : 2) : (gap[1] < gap[2] ? 1 : 2);
    float pa[3] = {p.x, p.y, p.z};
    float ea[3] = {extent.x, extent.y, extent.z};
    float n[3] = {0.0F, 0.0F, 0.0F};
    n[axis] = pa[axis] >= 0.0F ? 1.0F : -1.0F;
    float q[3] = {p.x, p.y, p.z};
    q[axis] = n[axis] * ea[axis];
    r.point = {q[0], q[1], q[2]};
    r.normal = {n[0], n[1], n[2]};
    r.distance = -gap[axis];
    return r;
}

// collider_shapes.h:68-74.
Surface closestOnPlane(V3 p) {
    Surface r;
    r.normal = {0.0F, 1.0F, 0.0F};
    r.point = {p.x, 0.0F, p.z};
    r.distance = p.y;
    return r;
}

// collider_shapes.h:77-82.
Surface closestOnCapsule(float radius, float halfHeight, V3 p) {
    V3 onSegment{0.0F, clampf(p.y, -halfHeight, halfHeight), 0.0F};
    Surface r = closestOnSphere(radius, sub(p, onSegment));
    r.point = add(r.point, onSegment);
    return r;
}

// collider_shapes.h:85-115.
Surface closestOnCylinder(float radius, float halfHeight, V3 p) {
    Surface r;
    V3 radial{p.x, 0.0F, p.z};
    float d = length(radial);
    V3 direction = d > 1.0e-6F ? divide(radial, d) : V3{1.0F, 0.0F, 0.0F};
    bool inside = std::fabs(p.y) <= halfHeight && d <= radius;
    if (inside) {
        float gapY = halfHeight - std::fabs(p.y);
        float gapR = radius - d;
        if (gapY < gapR) {
            float side = p.y >= 0.0F ? 1.0F : -1.0F;
            r.normal = {0.0F, side, 0.0F};
            r.point = {p.x, side * halfHeight, p.z};
            r.distance = -gapY;
        } else {
            r.normal = direction;
            r.point = add(scale(radius, direction), V3{0.0F, p.y, 0.0F});
            r.distance = -gapR;
        }
        return r;
    }
    V3 closest = scale(minf(d, radius), direction);
    closest.y = clampf(p.y, -halfHeight, halfHeight);
    V3 delta = sub(p, closest);
    float distance = length(delta);
    r.point = closest;
    r.normal = distance > 1.0e-6F ? divide(delta, distance) : V3{0.0F, 1.0F, 0.0F};
    r.distance = distance;
    return r;
}

// collider_shapes.h:118-134 (scene::ColliderShape: 0 sphere, 1 box, 2 plane,
// 3 cylinder, 4 capsule; a mesh falls through to a sphere of radius 0).
Surface closestOnColliderLocal(const sph_collider& c, V3 p) {
    float radius = c.data0[3];
    V3 half{c.data0[0], c.data0[1], c.data0[2]};
    switch (c.type) {
    case 0:
        return closestOnSphere(radius, p);
    case 1:
        return closestOnBox(half, p);
    case 2:
        return closestOnPlane(p);
    case 3:
        return closestOnCylinder(radius, half.y, p);
    case 4:
        return closestOnCapsule(radius, half.y, p);
    default:
        return closestOnSphere(0.0F, p);
    }
}

// glm mat4 * vec4(p, 1): (c0 x + c1 y) + (c2 z + c3 w), column-major.
inline V3 transformPoint(const float* m, V3 p) {
    float out[3];
    for (int r = 0; r < 3; ++r) {
        out[r] = (m[0 * 4 + r] * p.x + m[1 * 4 + r] * p.y) + (m[2 * 4 + r] * p.z + m[3 * 4 + r] * 1.0F);
    }
    return {out[0], out[1], out[2]};
}

// glm mat3(m) * vec3: (c0 x + c1 y) + c2 z.
inline V3 rotateVector(const float* m, V3 v) {
    float out[3];
    for (int r = 0; r < 3; ++r) {
        out[r] = (m[0 * 4 + r] * v.x + m[1 * 4 + r] * v.y) + m[2 * 4 + r] * v.z;
    }
    return {out[0], out[1], out[2]};
}

// glm::normalize: v * inversesqrt(dot(v, v)), inversesqrt(x) = 1 / sqrt(x).
inline V3 normalize(V3 v) { return scale(1.0F / std::sqrt(dot(v, v)), v); }

// fluid_sph.cpp:48-53.
inline void bounce(V3& velocity, V3 normal, float restitution) {
    float along = dot(velocity, normal);
    if (along < 0.0F) {
        velocity = sub(velocity, scale((1.0F + restitution) * along, normal));
    }
}

// fluid_sph.cpp:287-300: one-way push-out from every shape collider, in order.
void applyColliders(const sph_params& params, float radius, float restitution, V3& position, V3& velocity) {
    for (uint32_t c = 0; c < params.collider_count && c < SPH_MAX_COLLIDERS; ++c) {
        const sph_collider& collider = params.colliders[c];
        V3 local = transformPoint(collider.inverse_world, position);
        Surface surface = closestOnColliderLocal(collider, local);
        if (surface.distance < radius) {
            V3 normal = normalize(rotateVector(collider.world, surface.normal));
            position = add(transformPoint(collider.world, surface.point), scale(radius, normal));
            bounce(velocity, normal, restitution);
        }
    }
}

// A small persistent pool with the chunking of core::JobSystem::parallelFor
// (job_system.cpp:80-117): ranges of `GRANULARITY` ids, any worker may take
// any chunk. Results never depend on which worker ran a chunk.
class Pool {
public:
    explicit Pool(uint32_t threads) {
        for (uint32_t t = 1; t < threads; ++t) {
            workers.emplace_back([this] { loop(); });
        }
    }
    ~Pool() {
        {
            std::lock_guard<std::mutex> lock(mutex);
            stop = true;
            ++generation;
        }
        wake.notify_all();
        for (std::thread& w : workers) {
            w.join();
        }
    }
    uint32_t size() const { return static_cast<uint32_t>(workers.size()) + 1; }

    void parallelFor(uint32_t count, const std::function<void(uint32_t, uint32_t)>& body) {
        if (workers.empty() || count <= GRANULARITY) {
            body(0, count);
            return;
        }
        {
            std::lock_guard<std::mutex> lock(mutex);
            task = &body;
            total = count;
            next.store(0);
            active = static_cast<uint32_t>(workers.size());
            ++generation;
        }
        wake.notify_all();
        drain();
        std::unique_lock<std::mutex> lock(mutex);
        done.wait(lock, [this] { return active == 0; });
        task = nullptr;
    }

private:
    void drain() {
        for (;;) {
            uint32_t begin = next.fetch_add(GRANULARITY);
            if (begin >= total) {
                return;
            }
            (*task)(begin, std::min(begin + GRANULARITY, total));
        }
    }
    void loop() {
        uint64_t seen = 0;
        for (;;) {
            {
                std::unique_lock<std::mutex> lock(mutex);
                wake.wait(lock, [&] { return generation != seen; });
                seen = generation;
                if (stop) {
                    return;
                }
            }
            drain();
            {
                std::lock_guard<std::mutex> lock(mutex);
                if (--active == 0) {
                    done.notify_all();
                }
            }
        }
    }

    std::vector<std::thread> workers;
    std::mutex mutex;
    std::condition_variable wake;
    std::condition_variable done;
    const std::function<void(uint32_t, uint32_t)>* task = nullptr;
    std::atomic<uint32_t> next{0};
    uint32_t total = 0;
    uint32_t active = 0;
    uint64_t generation = 0;
    bool stop = false;
};

Pool& poolFor(uint32_t threads) {
    static std::mutex guard;
    static std::unique_ptr<Pool> pool;
    std::lock_guard<std::mutex> lock(guard);
    threads = std::max(threads, 1U);
    if (!pool || pool->size() != threads) {
        pool.reset();
        pool = std::make_unique<Pool>(threads);
    }
    return *pool;
}

// fluid_sph.cpp:55-61.
void forRange(uint32_t threads, uint32_t count, const std::function<void(uint32_t, uint32_t)>& body) {
    if (threads > 1 && count > GRANULARITY) {
        poolFor(threads).parallelFor(count, body);
    } else {
        body(0, count);
    }
}

struct Grid {
    std::vector<uint32_t> cellOf;
    std::vector<uint32_t> cellCounts;
    std::vector<uint32_t> cellParticles;
    uint32_t bucketCount(uint32_t b) const { return std::min(cellCounts[b], CAPACITY); }
    uint32_t particleAt(uint32_t b, uint32_t k) const { return cellParticles[static_cast<size_t>(b) * CAPACITY + k]; }
};

// fluid_sph.cpp:160-188.
void buildGrid(Grid& grid, const sph_params& params, const float* positions, uint32_t count, uint32_t threads) {
    uint32_t cells = params.lattice[3];
    float h = params.smoothing_radius;
    grid.cellCounts.assign(cells, 0U);
    grid.cellParticles.resize(static_cast<size_t>(cells) * CAPACITY);
    grid.cellOf.resize(count);
    forRange(threads, count, [&](uint32_t begin, uint32_t end) {
        for (uint32_t i = begin; i < end; ++i) {
            grid.cellOf[i] = spatialHash(spatialCell(xyz(positions + 4 * static_cast<size_t>(i)), h), cells);
        }
    });
    // Serial insert in ascending id: ids within a bucket stay ascending and
    // only the first CAPACITY are kept (fluid_sph.cpp:181-187).
    for (uint32_t i = 0; i < count; ++i) {
        uint32_t cell = grid.cellOf[i];
        uint32_t slot = grid.cellCounts[cell]++;
        if (slot < CAPACITY) {
            grid.cellParticles[static_cast<size_t>(cell) * CAPACITY + slot] = i;
        }
    }
}

bool validParams(const sph_params* params) {
    if (params == nullptr) {
        return false;
    }
    uint32_t cells = params->lattice[3];
    return cells != 0 && (cells & (cells - 1)) == 0 && params->smoothing_radius > 0.0F;
}

// fluid_sph.cpp:200-222.
void densityPass(const sph_params& params, const Grid& grid, float* pos, float* vel, uint32_t count, uint32_t threads) {
    float h = params.smoothing_radius;
    float mass = params.gravity[3];
    uint32_t cells = params.lattice[3];
    forRange(threads, count, [&](uint32_t begin, uint32_t end) {
        for (uint32_t i = begin; i < end; ++i) {
            V3 position = xyz(pos + 4 * static_cast<size_t>(i));
            Cell cell = spatialCell(position, h);
            float density = 0.0F;
            for (int dz = -1; dz <= 1; ++dz) {
                for (int dy = -1; dy <= 1; ++dy) {
                    for (int dx = -1; dx <= 1; ++dx) {
                        uint32_t bucket = spatialHash({cell.x + dx, cell.y + dy, cell.z + dz}, cells);
                        uint32_t n = grid.bucketCount(bucket);
                        for (uint32_t k = 0; k < n; ++k) {
                            uint32_t j = grid.particleAt(bucket, k);
                            V3 delta = sub(position, xyz(pos + 4 * static_cast<size_t>(j)));
                            density += mass * poly6(dot(delta, delta), h);
                        }
                    }
                }
            }
            density = std::max(density, 1e-6F);
            pos[4 * static_cast<size_t>(i) + 3] = density;
            vel[4 * static_cast<size_t>(i) + 3] = std::max(params.stiffness * (density - params.rest_density), 0.0F);
        }
    });
}

// fluid_sph.cpp:225-305.
void integratePass(const sph_params& params,
                   const Grid& grid,
                   const float* pos,
                   const float* vel,
                   float* nextPos,
                   float* nextVel,
                   uint32_t count,
                   float dt,
                   uint32_t threads) {
    float h = params.smoothing_radius;
    float mass = params.gravity[3];
    uint32_t cells = params.lattice[3];
    V3 gravity{params.gravity[0], params.gravity[1], params.gravity[2]};
    float radius = params.container_min[3];
    float restitution = params.container_max[3];
    forRange(threads, count, [&](uint32_t begin, uint32_t end) {
        for (uint32_t i = begin; i < end; ++i) {
            const float* self = pos + 4 * static_cast<size_t>(i);
            V3 position = xyz(self);
            float density = std::max(self[3], 1e-6F);
            V3 velocity = xyz(vel + 4 * static_cast<size_t>(i));
            float pressure = vel[4 * static_cast<size_t>(i) + 3];
            Cell cell = spatialCell(position, h);

            V3 force{0.0F, 0.0F, 0.0F};
            for (int dz = -1; dz <= 1; ++dz) {
                for (int dy = -1; dy <= 1; ++dy) {
                    for (int dx = -1; dx <= 1; ++dx) {
                        uint32_t bucket = spatialHash({cell.x + dx, cell.y + dy, cell.z + dz}, cells);
                        uint32_t n = grid.bucketCount(bucket);
                        for (uint32_t k = 0; k < n; ++k) {
                            uint32_t j = grid.particleAt(bucket, k);
                            if (j == i) {
                                continue;
                            }
                            const float* other = pos + 4 * static_cast<size_t>(j);
                            const float* otherVel = vel + 4 * static_cast<size_t>(j);
                            V3 delta = sub(position, xyz(other));
                            float distance = length(delta);
                            if (distance >= h || distance <= 1e-6F) {
                                continue;
                            }
                            float otherDensity = std::max(other[3], 1e-6F);
                            float pressureScale = -mass * (pressure + otherVel[3]) / (2.0F * otherDensity);
                            force = add(force, scale(pressureScale, spikyGradient(delta, distance, h)));
                            V3 viscous = divide(scale(params.viscosity * mass, sub(xyz(otherVel), velocity)), otherDensity);
                            float lap = viscosityLaplacian(distance, h);
                            force = add(force, {viscous.x * lap, viscous.y * lap, viscous.z * lap});
                        }
                    }
                }
            }

            V3 acceleration = add(add(divide(force, density), gravity), forceFieldsAcceleration(params, position));
            velocity = add(velocity, {acceleration.x * dt, acceleration.y * dt, acceleration.z * dt});
            float maxSpeed = 0.4F * h / dt;
            float speed = length(velocity);
            if (speed > maxSpeed) {
                float s = maxSpeed / speed;
                velocity = {velocity.x * s, velocity.y * s, velocity.z * s};
            }
            position = add(position, {velocity.x * dt, velocity.y * dt, velocity.z * dt});

            float p[3] = {position.x, position.y, position.z};
            float v[3] = {velocity.x, velocity.y, velocity.z};
            for (int axis = 0; axis < 3; ++axis) {
                float low = params.container_min[axis] + radius;
                float high = params.container_max[axis] - radius;
                if (p[axis] < low) {
                    p[axis] = low;
                    if (v[axis] < 0.0F) {
                        v[axis] = -v[axis] * restitution;
                    }
                } else if (p[axis] > high) {
                    p[axis] = high;
                    if (v[axis] > 0.0F) {
                        v[axis] = -v[axis] * restitution;
                    }
                }
            }
            position = {p[0], p[1], p[2]};
            velocity = {v[0], v[1], v[2]};
            applyColliders(params, radius, restitution, position, velocity);
            p[0] = position.x;
            p[1] = position.y;
            p[2] = position.z;
            v[0] = velocity.x;
            v[1] = velocity.y;
            v[2] = velocity.z;
            float* np = nextPos + 4 * static_cast<size_t>(i);
            float* nv = nextVel + 4 * static_cast<size_t>(i);
            np[0] = p[0];
            np[1] = p[1];
            np[2] = p[2];
            np[3] = density;
            nv[0] = v[0];
            nv[1] = v[1];
            nv[2] = v[2];
            nv[3] = pressure;
        }
    });
}

// ---- fluid surface (marching_cubes.cpp:18-24, :300-483; vertex_pack.h:38-51) ----

// The triangle table, derived from the rule the reference states for its
// MC_TABLE: a face's contour depends only on its four corner signs (an
// ambiguous face wraps each inside corner separately), each contour loop is
// traced from its lowest edge through the lower-numbered face first, turned
// to face outward, and fanned from its first edge; loops come out in order of
// their lowest edge.
struct McTable {
    int8_t entry[256][SPH_MC_TABLE_WIDTH];
};

const int MC_CORNER[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0}, {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
const int MC_EDGE[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {4, 5}, {5, 6}, {6, 7}, {7, 4}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};
const int MC_FACE[6][4] = {{0, 1, 2, 3}, {4, 5, 6, 7}, {0, 1, 5, 4}, {3, 2, 6, 7}, {0, 3, 7, 4}, {1, 2, 6, 5}};

int edgeBetween(int a, int b) {
    for (int e = 0; e < 12; ++e) {
        if ((MC_EDGE[e][0] == a && MC_EDGE[e][1] == b) || (MC_EDGE[e][0] == b && MC_EDGE[e][1] == a)) {
            return e;
        }
    }
    return -1;
}

McTable makeMcTable() {
    McTable table{};
    int faceEdge[6][4];
    for (int f = 0; f < 6; ++f) {
        for (int k = 0; k < 4; ++k) {
            faceEdge[f][k] = edgeBetween(MC_FACE[f][k], MC_FACE[f][(k + 1) % 4]);
        }
    }
    for (int code = 0; code < 256; ++code) {
        auto inside = [&](int c) { return ((code >> c) & 1) != 0; };
        bool active[12];
        for (int e = 0; e < 12; ++e) {
            active[e] = inside(MC_EDGE[e][0]) != inside(MC_EDGE[e][1]);
        }
        // Partner of edge e on face f: the next active edge walking from e
        // towards e's inside end.
        auto partner = [&](int f, int e) {
            int k = 0;
            while (faceEdge[f][k] != e) {
                ++k;
            }
            int step = inside(MC_FACE[f][(k + 1) % 4]) ? 1 : 3;
            int j = k;
            do {
                j = (j + step) % 4;
            } while (!active[faceEdge[f][j]]);
            return faceEdge[f][j];
        };
        auto facesOf = [&](int e, int* out) {
            int n = 0;
            for (int f = 0; f < 6; ++f) {
                for (int k = 0; k < 4; ++k) {
                    if (faceEdge[f][k] == e) {
                        out[n++] = f;
                    }
                }
            }
        };
        bool seen[12] = {};
        int written = 0;
        for (int e0 = 0; e0 < 12; ++e0) {
            if (!active[e0] || seen[e0]) {
                continue;
            }
            int loop[12];
            int length = 0;
            loop[length++] = e0;
            seen[e0] = true;
            int faces[2];
            facesOf(e0, faces);
            int face = std::min(faces[0], faces[1]);
            int e = partner(face, e0);
            while (e != e0) {
                loop[length++] = e;
                seen[e] = true;
                facesOf(e, faces);
                face = faces[0] == face ? faces[1] : faces[0];
                e = partner(face, e);
            }
            // Outward: the loop's area vector (edge midpoints) against the sum
            // of the inside-to-outside directions of its edges.
            double area[3] = {0, 0, 0};
            double out[3] = {0, 0, 0};
            for (int i = 0; i < length; ++i) {
                int a = loop[i];
                int b = loop[(i + 1) % length];
                double ma[3], mb[3];
                for (int d = 0; d < 3; ++d) {
                    ma[d] = 0.5 * (MC_CORNER[MC_EDGE[a][0]][d] + MC_CORNER[MC_EDGE[a][1]][d]);
                    mb[d] = 0.5 * (MC_CORNER[MC_EDGE[b][0]][d] + MC_CORNER[MC_EDGE[b][1]][d]);
                }
                area[0] += ma[1] * mb[2] - ma[2] * mb[1];
                area[1] += ma[2] * mb[0] - ma[0] * mb[2];
                area[2] += ma[0] * mb[1] - ma[1] * mb[0];
                int from = inside(MC_EDGE[a][0]) ? MC_EDGE[a][0] : MC_EDGE[a][1];
                int to = from == MC_EDGE[a][0] ? MC_EDGE[a][1] : MC_EDGE[a][0];
                for (int d = 0; d < 3; ++d) {
                    out[d] += MC_CORNER[to][d] - MC_CORNER[from][d];
                }
            }
            if (area[0] * out[0] + area[1] * out[1] + area[2] * out[2] < 0.0) {
                std::reverse(loop, loop + length);
            }
            for (int i = 1; i + 1 < length; ++i) {
                table.entry[code][written++] = static_cast<int8_t>(loop[0]);
                table.entry[code][written++] = static_cast<int8_t>(loop[i]);
                table.entry[code][written++] = static_cast<int8_t>(loop[i + 1]);
            }
        }
        for (int i = written; i < static_cast<int>(SPH_MC_TABLE_WIDTH); ++i) {
            table.entry[code][i] = -1;
        }
    }
    return table;
}

const McTable& mcTable() {
    static const McTable table = makeMcTable();
    return table;
}

// marching_cubes.cpp:312-347 (sampleField): 27 buckets in (z, y, x) order,
// a bucket already visited (two neighbour cells that hash alike) skipped.
float sampleField(const float* positions, const Grid& grid, uint32_t cells, V3 point, float radius) {
    float radiusSq = radius * radius;
    float total = 0.0F;
    Cell base = spatialCell(point, radius);
    uint32_t visited[27];
    uint32_t visitedCount = 0;
    for (int z = -1; z <= 1; ++z) {
        for (int y = -1; y <= 1; ++y) {
            for (int x = -1; x <= 1; ++x) {
                uint32_t bucket = spatialHash({base.x + x, base.y + y, base.z + z}, cells);
                if (std::find(visited, visited + visitedCount, bucket) != visited + visitedCount) {
                    continue;
                }
                visited[visitedCount++] = bucket;
                uint32_t n = grid.bucketCount(bucket);
                for (uint32_t k = 0; k < n; ++k) {
                    V3 delta = sub(xyz(positions + 4 * static_cast<size_t>(grid.particleAt(bucket, k))), point);
                    float distanceSq = dot(delta, delta);
                    if (distanceSq >= radiusSq) {
                        continue;
                    }
                    float d = 1.0F - distanceSq / radiusSq;
                    total += d * d * d;
                }
            }
        }
    }
    return total;
}

// marching_cubes.cpp:350-359 (fieldAt): 0 outside the sample grid.
inline float fieldAt(const float* field, uint32_t samples, int x, int y, int z) {
    int s = static_cast<int>(samples);
    if (x < 0 || y < 0 || z < 0 || x >= s || y >= s || z >= s) {
        return 0.0F;
    }
    return field[(static_cast<size_t>(z) * samples + static_cast<size_t>(y)) * samples + static_cast<size_t>(x)];
}

// vertex_pack.h:20-28, :38-51 (packSnorm2x16, packUnitVector).
inline uint32_t quantizeSnorm16(float x) {
    auto q = static_cast<int32_t>(std::lround(std::clamp(x, -1.0F, 1.0F) * 32767.0F));
    return static_cast<uint32_t>(q) & 0xFFFFU;
}

inline float signNotZero(float v) { return v >= 0.0F ? 1.0F : -1.0F; }

uint32_t packUnitVector(V3 n) {
    float sum = std::fabs(n.x) + std::fabs(n.y) + std::fabs(n.z);
    if (sum <= 0.0F) {
        return quantizeSnorm16(0.0F) | (quantizeSnorm16(0.0F) << 16U);
    }
    n = divide(n, sum);
    float px = n.x;
    float py = n.y;
    if (n.z < 0.0F) {
        px = (1.0F - std::fabs(n.y)) * signNotZero(n.x);
        py = (1.0F - std::fabs(n.x)) * signNotZero(n.y);
    }
    return quantizeSnorm16(px) | (quantizeSnorm16(py) << 16U);
}

} // namespace

extern "C" {

int oracle_abi(void) { return SPH_ABI_VERSION; }

uint32_t oracle_spatial_hash(int32_t cx, int32_t cy, int32_t cz, uint32_t cell_count) {
    return spatialHash({cx, cy, cz}, cell_count);
}

void oracle_spatial_cell(const float position[3], float cell_size, int32_t out[3]) {
    Cell c = spatialCell({position[0], position[1], position[2]}, cell_size);
    out[0] = c.x;
    out[1] = c.y;
    out[2] = c.z;
}

// fluid_sph.cpp:65-100 (colliders and force fields come from a scene; none here).
int oracle_derive_params(const sph_fluid_settings* settings,
                         const float emitter_world[16],
                         uint32_t particle_count,
                         uint32_t cell_count,
                         sph_params* out) {
    if (settings == nullptr || emitter_world == nullptr || out == nullptr) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    std::memset(out, 0, sizeof(*out));
    float spacing = settings->particle_radius * 2.0F;
    std::memcpy(out->emitter_world, emitter_world, sizeof(out->emitter_world));
    for (int a = 0; a < 3; ++a) {
        out->emitter_half_extents[a] = settings->emitter_half_extents[a];
        out->container_min[a] = settings->container_min[a];
        out->container_max[a] = settings->container_max[a];
        out->gravity[a] = settings->gravity[a];
    }
    out->emitter_half_extents[3] = spacing;
    out->container_min[3] = settings->particle_radius;
    out->container_max[3] = 0.3F;
    out->gravity[3] = settings->rest_density * spacing * spacing * spacing;
    out->smoothing_radius = std::max(settings->smoothing_radius, spacing);
    out->rest_density = settings->rest_density;
    out->stiffness = settings->stiffness;
    out->viscosity = settings->viscosity;
    auto along = [spacing](float half) {
        return std::max(1U, static_cast<uint32_t>(std::floor(half * 2.0F / spacing)));
    };
    uint32_t nx = along(settings->emitter_half_extents[0]);
    uint32_t ny = along(settings->emitter_half_extents[1]);
    uint32_t nz = std::max(1U, (particle_count + nx * ny - 1) / (nx * ny));
    out->lattice[0] = nx;
    out->lattice[1] = ny;
    out->lattice[2] = nz;
    out->lattice[3] = cell_count;
    return SPH_OK;
}

// fluid_sph.cpp:128-136.
uint32_t oracle_fluid_substeps(const sph_params* params, float delta_seconds) {
    float h = params->smoothing_radius;
    float gravity = std::max(length({params->gravity[0], params->gravity[1], params->gravity[2]}), 0.1F);
    float stable = std::min(0.4F * h / std::sqrt(std::max(params->stiffness, 1.0F)), 0.25F * std::sqrt(h / gravity));
    float frameStep = std::min(std::max(delta_seconds, 0.0F), SPH_MAX_FRAME_STEP);
    auto steps = static_cast<uint32_t>(std::ceil(frameStep / std::max(stable, 1e-5F)));
    return std::clamp(steps, 1U, 8U);
}

// fluid_sph.cpp:138-154. glm's mat4 * vec4 sums the columns as
// (c0*x + c1*y) + (c2*z + c3*w).
void oracle_emit(const sph_params* params, uint32_t count, float* positions, float* velocities) {
    uint32_t cx = std::max(params->lattice[0], 1U);
    uint32_t cy = std::max(params->lattice[1], 1U);
    uint32_t cz = std::max(params->lattice[2], 1U);
    float spacing = params->emitter_half_extents[3];
    float extent[3] = {static_cast<float>(cx - 1U) * spacing * 0.5F, static_cast<float>(cy - 1U) * spacing * 0.5F,
                       static_cast<float>(cz - 1U) * spacing * 0.5F};
    const float* m = params->emitter_world;
    for (uint32_t i = 0; i < count; ++i) {
        uint32_t index[3] = {i % cx, (i / cx) % cy, i / (cx * cy)};
        float local[4];
        for (int a = 0; a < 3; ++a) {
            local[a] = static_cast<float>(index[a]) * spacing - extent[a];
        }
        local[3] = 1.0F;
        float* p = positions + 4 * static_cast<size_t>(i);
        for (int r = 0; r < 3; ++r) {
            float add0 = m[0 * 4 + r] * local[0] + m[1 * 4 + r] * local[1];
            float add1 = m[2 * 4 + r] * local[2] + m[3 * 4 + r] * local[3];
            p[r] = add0 + add1;
        }
        p[3] = params->rest_density;
        if (velocities != nullptr) {
            float* v = velocities + 4 * static_cast<size_t>(i);
            v[0] = v[1] = v[2] = v[3] = 0.0F;
        }
    }
}

int oracle_grid_build(const sph_params* params,
                      const float* positions,
                      uint32_t count,
                      uint32_t* cell_of,
                      uint32_t* cell_counts,
                      uint32_t* cell_particles,
                      uint32_t threads) {
    if (!validParams(params) || (count > 0 && positions == nullptr)) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    Grid grid;
    buildGrid(grid, *params, positions, count, threads);
    if (cell_of != nullptr) {
        std::memcpy(cell_of, grid.cellOf.data(), grid.cellOf.size() * sizeof(uint32_t));
    }
    if (cell_counts != nullptr) {
        std::memcpy(cell_counts, grid.cellCounts.data(), grid.cellCounts.size() * sizeof(uint32_t));
    }
    if (cell_particles != nullptr) {
        uint32_t cells = params->lattice[3];
        for (uint32_t b = 0; b < cells; ++b) {
            uint32_t n = grid.bucketCount(b);
            for (uint32_t k = 0; k < n; ++k) {
                cell_particles[static_cast<size_t>(b) * CAPACITY + k] = grid.particleAt(b, k);
            }
        }
    }
    return SPH_OK;
}

int oracle_density(const sph_params* params, float* positions, float* velocities, uint32_t count, uint32_t threads) {
    if (!validParams(params)) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    Grid grid;
    buildGrid(grid, *params, positions, count, threads);
    densityPass(*params, grid, positions, velocities, count, threads);
    return SPH_OK;
}

// fluid_sph.cpp:190-309.
int oracle_substep(const sph_params* params, float* positions, float* velocities, uint32_t count, float dt, uint32_t threads) {
    if (!validParams(params)) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    if (count == 0) {
        return SPH_OK;
    }
    Grid grid;
    buildGrid(grid, *params, positions, count, threads);
    densityPass(*params, grid, positions, velocities, count, threads);
    std::vector<float> nextPos(4 * static_cast<size_t>(count));
    std::vector<float> nextVel(4 * static_cast<size_t>(count));
    integratePass(*params, grid, positions, velocities, nextPos.data(), nextVel.data(), count, dt, threads);
    std::memcpy(positions, nextPos.data(), nextPos.size() * sizeof(float));
    std::memcpy(velocities, nextVel.data(), nextVel.size() * sizeof(float));
    return SPH_OK;
}

// fluid_sph.cpp:311-321.
int oracle_step(const sph_params* params,
                float* positions,
                float* velocities,
                uint32_t count,
                float delta_seconds,
                uint32_t threads) {
    if (!validParams(params)) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    if (count == 0 || delta_seconds <= 0.0F) {
        return SPH_OK;
    }
    uint32_t substeps = oracle_fluid_substeps(params, delta_seconds);
    float frameStep = std::min(delta_seconds, SPH_MAX_FRAME_STEP);
    float dt = frameStep / static_cast<float>(substeps);
    for (uint32_t s = 0; s < substeps; ++s) {
        int status = oracle_substep(params, positions, velocities, count, dt, threads);
        if (status != SPH_OK) {
            return status;
        }
    }
    return SPH_OK;
}

int oracle_pair_counts(const sph_params* params,
                       const float* positions,
                       uint32_t count,
                       uint64_t* candidates,
                       uint64_t* in_range,
                       uint32_t threads) {
    if (!validParams(params)) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    Grid grid;
    buildGrid(grid, *params, positions, count, threads);
    float h = params->smoothing_radius;
    float h2 = h * h;
    uint32_t cells = params->lattice[3];
    std::atomic<uint64_t> p{0};
    std::atomic<uint64_t> q{0};
    forRange(threads, count, [&](uint32_t begin, uint32_t end) {
        uint64_t lp = 0;
        uint64_t lq = 0;
        for (uint32_t i = begin; i < end; ++i) {
            V3 position = xyz(positions + 4 * static_cast<size_t>(i));
            Cell cell = spatialCell(position, h);
            for (int dz = -1; dz <= 1; ++dz) {
                for (int dy = -1; dy <= 1; ++dy) {
                    for (int dx = -1; dx <= 1; ++dx) {
                        uint32_t bucket = spatialHash({cell.x + dx, cell.y + dy, cell.z + dz}, cells);
                        uint32_t n = grid.bucketCount(bucket);
                        lp += n;
                        for (uint32_t k = 0; k < n; ++k) {
                            V3 delta = sub(position, xyz(positions + 4 * static_cast<size_t>(grid.particleAt(bucket, k))));
                            lq += dot(delta, delta) < h2 ? 1 : 0;
                        }
                    }
                }
            }
        }
        p += lp;
        q += lq;
    });
    if (candidates != nullptr) {
        *candidates = p.load();
    }
    if (in_range != nullptr) {
        *in_range = q.load();
    }
    return SPH_OK;
}

int oracle_stats(const sph_params* params, const float* positions, const float* velocities, uint32_t count, sph_stats* out) {
    if (params == nullptr || out == nullptr) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    std::memset(out, 0, sizeof(*out));
    out->particles = count;
    out->buckets = params->lattice[3];
    double rho0 = params->rest_density;
    double mass = params->gravity[3];
    double sumRho = 0.0;
    double sumCompression = 0.0;
    double maxRho = 0.0;
    double com[3] = {0.0, 0.0, 0.0};
    double kinetic = 0.0;
    uint32_t nonfinite = 0;
    for (uint32_t i = 0; i < count; ++i) {
        const float* p = positions + 4 * static_cast<size_t>(i);
        const float* v = velocities + 4 * static_cast<size_t>(i);
        bool finite = std::isfinite(p[0]) && std::isfinite(p[1]) && std::isfinite(p[2]) && std::isfinite(v[0]) &&
                      std::isfinite(v[1]) && std::isfinite(v[2]);
        nonfinite += finite ? 0 : 1;
        double rho = p[3];
        sumRho += rho;
        sumCompression += std::max(0.0, rho - rho0) / rho0;
        maxRho = std::max(maxRho, rho);
        for (int a = 0; a < 3; ++a) {
            com[a] += p[a];
        }
        kinetic += 0.5 * mass * (static_cast<double>(v[0]) * v[0] + static_cast<double>(v[1]) * v[1] +
                                 static_cast<double>(v[2]) * v[2]);
    }
    if (count > 0) {
        out->mean_density = sumRho / count;
        out->mean_compression = sumCompression / count;
        for (int a = 0; a < 3; ++a) {
            out->centre_of_mass[a] = com[a] / count;
        }
    }
    out->max_density = maxRho;
    out->kinetic_energy = kinetic;
    out->nonfinite = nonfinite;
    return SPH_OK;
}

void oracle_mc_table(int8_t* out) {
    std::memcpy(out, mcTable().entry, sizeof(McTable::entry));
}

// marching_cubes.cpp:363-395 (buildFluidField).
int oracle_surface_field(const sph_params* params, const float* positions, uint32_t count, uint32_t resolution,
                         uint32_t threads, float* field) {
    if (!validParams(params) || resolution == 0 || field == nullptr) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    uint32_t samples = resolution + 1;
    size_t total = static_cast<size_t>(samples) * samples * samples;
    std::fill(field, field + total, 0.0F);
    if (count == 0) {
        return SPH_OK;
    }
    Grid grid;
    buildGrid(grid, *params, positions, count, threads);
    V3 origin{params->container_min[0], params->container_min[1], params->container_min[2]};
    V3 span = sub({params->container_max[0], params->container_max[1], params->container_max[2]}, origin);
    V3 cell = divide(span, static_cast<float>(resolution));
    float radius = params->smoothing_radius;
    uint32_t cells = params->lattice[3];
    forRange(threads, static_cast<uint32_t>(total), [&](uint32_t begin, uint32_t end) {
        for (uint32_t i = begin; i < end; ++i) {
            uint32_t x = i % samples;
            uint32_t y = (i / samples) % samples;
            uint32_t z = i / (samples * samples);
            if (x == 0 || y == 0 || z == 0 || x == resolution || y == resolution || z == resolution) {
                continue;
            }
            V3 point = add(origin, V3{static_cast<float>(x) * cell.x, static_cast<float>(y) * cell.y,
                                      static_cast<float>(z) * cell.z});
            field[i] = sampleField(positions, grid, cells, point, radius);
        }
    });
    return SPH_OK;
}

// marching_cubes.cpp:397-481 (marchFluidField), in serial cell order.
int oracle_march_field(const float* field, uint32_t resolution, const float origin[3], const float cell[3], float iso,
                       sph_surface_vertex* out, uint32_t capacity, uint32_t* written) {
    if (field == nullptr || written == nullptr || resolution == 0) {
        return SPH_ERR_INVALID_ARGUMENT;
    }
    *written = 0;
    if (capacity < 3) {
        return SPH_OK;
    }
    const McTable& table = mcTable();
    uint32_t samples = resolution + 1;
    V3 o{origin[0], origin[1], origin[2]};
    V3 c{cell[0], cell[1], cell[2]};
    uint32_t slot = 0;
    uint32_t cells = resolution * resolution * resolution;
    for (uint32_t i = 0; i < cells; ++i) {
        int base[3] = {static_cast<int>(i % resolution), static_cast<int>((i / resolution) % resolution),
                       static_cast<int>(i / (resolution * resolution))};
        float values[8];
        uint32_t code = 0;
        for (int k = 0; k < 8; ++k) {
            values[k] = fieldAt(field, samples, base[0] + MC_CORNER[k][0], base[1] + MC_CORNER[k][1],
                                base[2] + MC_CORNER[k][2]);
            if (values[k] >= iso) {
                code |= 1U << k;
            }
        }
        const int8_t* entry = table.entry[code];
        if (entry[0] < 0) {
            continue;
        }
        uint32_t vertices = 0;
        while (vertices < SPH_MC_TABLE_WIDTH && entry[vertices] >= 0) {
            ++vertices;
        }
        if (slot + vertices > capacity) {
            break;  // every later cell's slot lies past this one's
        }
        for (uint32_t v = 0; v < vertices; ++v) {
            int edge = entry[v];
            int a = MC_EDGE[edge][0];
            int b = MC_EDGE[edge][1];
            float va = values[a];
            float vb = values[b];
            float t = std::fabs(vb - va) > 1.0e-8F ? (iso - va) / (vb - va) : 0.5F;
            t = clampf(t, 0.0F, 1.0F);
            int ca[3], cb[3];
            for (int d = 0; d < 3; ++d) {
                ca[d] = base[d] + MC_CORNER[a][d];
                cb[d] = base[d] + MC_CORNER[b][d];
            }
            V3 pa = add(o, V3{static_cast<float>(ca[0]) * c.x, static_cast<float>(ca[1]) * c.y,
                              static_cast<float>(ca[2]) * c.z});
            V3 pb = add(o, V3{static_cast<float>(cb[0]) * c.x, static_cast<float>(cb[1]) * c.y,
                              static_cast<float>(cb[2]) * c.z});
            V3 d = sub(pb, pa);
            V3 point = add(pa, V3{d.x * t, d.y * t, d.z * t});
            auto gradient = [&](const int* p) {
                V3 g{fieldAt(field, samples, p[0] + 1, p[1], p[2]) - fieldAt(field, samples, p[0] - 1, p[1], p[2]),
                     fieldAt(field, samples, p[0], p[1] + 1, p[2]) - fieldAt(field, samples, p[0], p[1] - 1, p[2]),
                     fieldAt(field, samples, p[0], p[1], p[2] + 1) - fieldAt(field, samples, p[0], p[1], p[2] - 1)};
                return V3{g.x / c.x, g.y / c.y, g.z / c.z};
            };
            V3 ga = gradient(ca);
            V3 gb = gradient(cb);
            V3 dg = sub(gb, ga);
            V3 n = add(ga, V3{dg.x * t, dg.y * t, dg.z * t});
            n = {-n.x, -n.y, -n.z};
            if (!(length(n) > 1.0e-12F)) {
                n = {0.0F, 1.0F, 0.0F};
            }
            float inv = 1.0F / std::sqrt(dot(n, n));
            n = {n.x * inv, n.y * inv, n.z * inv};
            out[slot + v].position[0] = point.x;
            out[slot + v].position[1] = point.y;
            out[slot + v].position[2] = point.z;
            out[slot + v].normal = packUnitVector(n);
        }
        slot += vertices;
    }
    *written = slot;
    return SPH_OK;
}

// fluid.cpp:402-466. glm::scale(glm::translate(I, p), vec3{r}) has the
// radius on the diagonal and the position in column 3; the TLAS transform is
// that matrix's first three rows (row-major), as the reference copies it.
int oracle_write_instances(const float* pos, const float* prev, uint32_t n, float radius, sph_instance* instances,
                           uint32_t instance_base, uint32_t sphere_mesh, sph_tlas_instance* tlas, uint32_t tlas_base,
                           uint64_t blas, uint32_t fluid_index, uint32_t flags, uint32_t threads) {
    if (n == 0) {
        return 0;
    }
    if (pos == nullptr || instances == nullptr || (prev == nullptr && (flags & SPH_INSTANCES_RESET_HISTORY) == 0) ||
        ((flags & SPH_INSTANCES_WRITE_TLAS) != 0 && tlas == nullptr)) {
        return 1;
    }
    const bool history = (flags & SPH_INSTANCES_RESET_HISTORY) == 0;
    const bool write_tlas = (flags & SPH_INSTANCES_WRITE_TLAS) != 0;
    const bool surface = (flags & SPH_INSTANCES_SURFACE_TLAS) != 0;
    auto model = [radius](const float* p, float out[16]) {
        for (int k = 0; k < 16; ++k) {
            out[k] = 0.0F;
        }
        out[0] = radius;
        out[5] = radius;
        out[10] = radius;
        out[12] = p[0];
        out[13] = p[1];
        out[14] = p[2];
        out[15] = 1.0F;
    };
    if (write_tlas && surface) {
        // The surface record first, every other record inactive (all zero).
        std::memset(tlas + tlas_base, 0, sizeof(sph_tlas_instance) * n);
        sph_tlas_instance& entry = tlas[tlas_base];
        entry.transform[0] = 1.0F;
        entry.transform[5] = 1.0F;
        entry.transform[10] = 1.0F;
        entry.custom_index_mask = (SPH_FLUID_SURFACE_CUSTOM_INDEX | fluid_index) | (SPH_FLUID_SURFACE_RAY_MASK << 24U);
        entry.sbt_offset_flags = 1U << 24U;  // VK_GEOMETRY_INSTANCE_TRIANGLE_FACING_CULL_DISABLE_BIT_KHR
        entry.blas = blas;
    }
    Pool pool(std::max(1U, threads));
    pool.parallelFor(n, [&](uint32_t begin, uint32_t end) {
        for (uint32_t i = begin; i < end; ++i) {
            const float* p = pos + 4 * static_cast<size_t>(i);
            const float* q = history ? prev + 4 * static_cast<size_t>(i) : p;
            const uint32_t slot = instance_base + i;
            sph_instance& out = instances[slot];
            model(p, out.model);
            model(q, out.previous_model);
            for (int k = 0; k < 16; ++k) {
                out.normal_matrix[k] = (k % 5 == 0) ? 1.0F : 0.0F;
            }
            out.mesh_index = sphere_mesh;
            out.bucket = 0;
            out.bucket_base = 0;
            out.joint_offset = SPH_NO_JOINTS;
            out.skinned_vertex_offset = SPH_NO_JOINTS;
            out.previous_skinned_vertex_offset = SPH_NO_JOINTS;
            out.skinned_meshlet_offset = 0;
            out.visibility_base = 0;
            if (write_tlas && !surface) {
                sph_tlas_instance entry{};
                for (int row = 0; row < 3; ++row) {
                    for (int column = 0; column < 4; ++column) {
                        entry.transform[row * 4 + column] = out.model[column * 4 + row];
                    }
                }
                entry.custom_index_mask = (slot & 0xFFFFFFU) | (0xFFU << 24U);
                entry.sbt_offset_flags = 0;
                entry.blas = blas;
                tlas[tlas_base + i] = entry;
            }
        }
    });
    return 0;
}

uint32_t oracle_hardware_threads(void) { return std::max(1U, std::thread::hardware_concurrency()); }

} // extern "C"
