// glm_shim.hpp — a minimal stand-in for the parts of glm the reference's
// fluid solver uses, so that the unmodified sources of
// src/physics/fluid_sph.cpp and src/core/job_system.cpp compile here (glm is
// not installed). TEST INFRASTRUCTURE ONLY: it builds the reference checker
// under oracle/_ref.
//
// Written from glm's documented semantics, not from its sources. The
// properties the bit-exact comparison relies on:
//   - every vector operator is component-wise with one rounding per component
//     (vec / scalar divides each component; it does not multiply by 1/s);
//   - dot(a, b) of vec3 is (a.x*b.x + a.y*b.y) + a.z*b.z, left to right;
//   - length(v) is sqrt(dot(v, v));
//   - mat4 * vec4 sums the scaled columns as (c0*x + c1*y) + (c2*z + c3*w).
// glm itself cannot be consulted here, so these orders are an assumption
// that the restatement in oracle/sph_oracle.cpp shares.
#pragma once

#include <cmath>
#include <cstddef>
#include <cstdint>

namespace glm {

template <int L, typename T> struct vec;

template <typename T> struct vec<2, T> {
    T x, y;
    constexpr vec() : x(0), y(0) {}
    constexpr explicit vec(T s) : x(s), y(s) {}
    constexpr vec(T a, T b) : x(a), y(b) {}
    T& operator[](int i) { return (&x)[i]; }
    const T& operator[](int i) const { return (&x)[i]; }
    bool operator==(const vec&) const = default;
};

template <typename T> struct vec<3, T> {
    T x, y, z;
    constexpr vec() : x(0), y(0), z(0) {}
    constexpr explicit vec(T s) : x(s), y(s), z(s) {}
    constexpr vec(T a, T b, T c) : x(a), y(b), z(c) {}
    // glm's vec(X, Y, Z): each component converted on its own.
    template <typename A, typename B, typename C>
    constexpr vec(A a, B b, C c) : x(static_cast<T>(a)), y(static_cast<T>(b)), z(static_cast<T>(c)) {}
    template <typename U> constexpr explicit vec(const vec<3, U>& v)
        : x(static_cast<T>(v.x)), y(static_cast<T>(v.y)), z(static_cast<T>(v.z)) {}
    template <typename U> constexpr explicit vec(const vec<4, U>& v)
        : x(static_cast<T>(v.x)), y(static_cast<T>(v.y)), z(static_cast<T>(v.z)) {}
    T& operator[](int i) { return (&x)[i]; }
    const T& operator[](int i) const { return (&x)[i]; }
    vec& operator+=(const vec& o) { x += o.x; y += o.y; z += o.z; return *this; }
    vec& operator-=(const vec& o) { x -= o.x; y -= o.y; z -= o.z; return *this; }
    vec& operator*=(T s) { x *= s; y *= s; z *= s; return *this; }
    vec& operator/=(T s) { x /= s; y /= s; z /= s; return *this; }
    bool operator==(const vec&) const = default;
};

template <typename T> struct vec<4, T> {
    T x, y, z, w;
    constexpr vec() : x(0), y(0), z(0), w(0) {}
    constexpr explicit vec(T s) : x(s), y(s), z(s), w(s) {}
    constexpr vec(T a, T b, T c, T d) : x(a), y(b), z(c), w(d) {}
    constexpr vec(const vec<3, T>& v, T d) : x(v.x), y(v.y), z(v.z), w(d) {}
    template <typename U> constexpr explicit vec(const vec<4, U>& v)
        : x(static_cast<T>(v.x)), y(static_cast<T>(v.y)), z(static_cast<T>(v.z)), w(static_cast<T>(v.w)) {}
    T& operator[](int i) { return (&x)[i]; }
    const T& operator[](int i) const { return (&x)[i]; }
    bool operator==(const vec&) const = default;
};

using vec2 = vec<2, float>;
using vec3 = vec<3, float>;
using vec4 = vec<4, float>;
using ivec3 = vec<3, int32_t>;
using uvec3 = vec<3, uint32_t>;
using uvec4 = vec<4, uint32_t>;

// ---- component-wise arithmetic --------------------------------------------
#define GLM_SHIM_BINOP(OP)                                                                                       \
    template <typename T> constexpr vec<3, T> operator OP(const vec<3, T>& a, const vec<3, T>& b) {             \
        return vec<3, T>(a.x OP b.x, a.y OP b.y, a.z OP b.z);                                                    \
    }                                                                                                            \
    template <typename T> constexpr vec<3, T> operator OP(const vec<3, T>& a, T s) {                            \
        return vec<3, T>(a.x OP s, a.y OP s, a.z OP s);                                                          \
    }                                                                                                            \
    template <typename T> constexpr vec<3, T> operator OP(T s, const vec<3, T>& a) {                            \
        return vec<3, T>(s OP a.x, s OP a.y, s OP a.z);                                                          \
    }                                                                                                            \
    template <typename T> constexpr vec<4, T> operator OP(const vec<4, T>& a, const vec<4, T>& b) {             \
        return vec<4, T>(a.x OP b.x, a.y OP b.y, a.z OP b.z, a.w OP b.w);                                        \
    }                                                                                                            \
    template <typename T> constexpr vec<4, T> operator OP(const vec<4, T>& a, T s) {                            \
        return vec<4, T>(a.x OP s, a.y OP s, a.z OP s, a.w OP s);                                                \
    }                                                                                                            \
    template <typename T> constexpr vec<4, T> operator OP(T s, const vec<4, T>& a) {                            \
        return vec<4, T>(s OP a.x, s OP a.y, s OP a.z, s OP a.w);                                                \
    }
GLM_SHIM_BINOP(+)
GLM_SHIM_BINOP(-)
GLM_SHIM_BINOP(*)
GLM_SHIM_BINOP(/)
#undef GLM_SHIM_BINOP

template <typename T> constexpr vec<2, T> operator-(T s, const vec<2, T>& a) { return vec<2, T>(s - a.x, s - a.y); }
template <typename T> constexpr vec<2, T> operator*(const vec<2, T>& a, const vec<2, T>& b) {
    return vec<2, T>(a.x * b.x, a.y * b.y);
}
template <typename T> constexpr vec<3, T> operator-(const vec<3, T>& a) { return vec<3, T>(-a.x, -a.y, -a.z); }
template <typename T> constexpr vec<4, T> operator-(const vec<4, T>& a) { return vec<4, T>(-a.x, -a.y, -a.z, -a.w); }

// ---- common ----------------------------------------------------------------
inline vec3 floor(const vec3& v) { return vec3(std::floor(v.x), std::floor(v.y), std::floor(v.z)); }
inline vec3 abs(const vec3& v) { return vec3(std::fabs(v.x), std::fabs(v.y), std::fabs(v.z)); }
inline vec2 abs(const vec2& v) { return vec2(std::fabs(v.x), std::fabs(v.y)); }
template <typename T> constexpr T shim_min(T a, T b) { return b < a ? b : a; }
template <typename T> constexpr T shim_max(T a, T b) { return a < b ? b : a; }
template <typename T> constexpr vec<3, T> max(const vec<3, T>& a, const vec<3, T>& b) {
    return vec<3, T>(shim_max(a.x, b.x), shim_max(a.y, b.y), shim_max(a.z, b.z));
}
template <typename T> constexpr vec<3, T> min(const vec<3, T>& a, const vec<3, T>& b) {
    return vec<3, T>(shim_min(a.x, b.x), shim_min(a.y, b.y), shim_min(a.z, b.z));
}
template <typename T> constexpr vec<3, T> clamp(const vec<3, T>& v, const vec<3, T>& lo, const vec<3, T>& hi) {
    return min(max(v, lo), hi);
}

// ---- geometric -------------------------------------------------------------
inline float dot(const vec3& a, const vec3& b) {
    vec3 t = a * b;
    return t.x + t.y + t.z;
}
inline float length(const vec3& v) { return std::sqrt(dot(v, v)); }
inline float length2(const vec3& v) { return dot(v, v); }
inline float distance(const vec3& a, const vec3& b) { return length(b - a); }
inline vec3 normalize(const vec3& v) { return v * (1.0F / std::sqrt(dot(v, v))); }
inline vec3 cross(const vec3& a, const vec3& b) {
    return vec3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}

// ---- matrices (column-major) ------------------------------------------------
struct mat4;

struct mat3 {
    vec3 c[3];
    mat3() : c{vec3(1, 0, 0), vec3(0, 1, 0), vec3(0, 0, 1)} {}
    explicit mat3(float s) : c{vec3(s, 0, 0), vec3(0, s, 0), vec3(0, 0, s)} {}
    explicit mat3(const mat4& m);
    vec3& operator[](int i) { return c[i]; }
    const vec3& operator[](int i) const { return c[i]; }
};

inline vec3 operator*(const mat3& m, const vec3& v) { return (m[0] * v.x + m[1] * v.y) + m[2] * v.z; }

struct mat4 {
    vec4 c[4];
    mat4() : c{vec4(1, 0, 0, 0), vec4(0, 1, 0, 0), vec4(0, 0, 1, 0), vec4(0, 0, 0, 1)} {}
    explicit mat4(float s) : c{vec4(s, 0, 0, 0), vec4(0, s, 0, 0), vec4(0, 0, s, 0), vec4(0, 0, 0, s)} {}
    vec4& operator[](int i) { return c[i]; }
    const vec4& operator[](int i) const { return c[i]; }
    bool operator==(const mat4& o) const {
        return c[0] == o.c[0] && c[1] == o.c[1] && c[2] == o.c[2] && c[3] == o.c[3];
    }
};

inline mat3::mat3(const mat4& m) : c{vec3(m[0]), vec3(m[1]), vec3(m[2])} {}

inline vec4 operator*(const mat4& m, const vec4& v) {
    vec4 add0 = m[0] * v.x + m[1] * v.y;
    vec4 add1 = m[2] * v.z + m[3] * v.w;
    return add0 + add1;
}

inline mat4 operator*(const mat4& a, const mat4& b) {
    mat4 r;
    for (int i = 0; i < 4; ++i) {
        r[i] = a * b[i];
    }
    return r;
}

inline mat4 translate(const mat4& m, const vec3& t) {
    mat4 r = m;
    r[3] = m[0] * t.x + m[1] * t.y + m[2] * t.z + m[3];
    return r;
}

// General 4x4 inverse by cofactors. Only collectShapeColliders calls it, and
// no checker path does.
inline mat4 inverse(const mat4& m) {
    float a[16];
    for (int col = 0; col < 4; ++col) {
        for (int row = 0; row < 4; ++row) {
            a[col * 4 + row] = m[col][row];
        }
    }
    float inv[16];
    inv[0] = a[5] * a[10] * a[15] - a[5] * a[11] * a[14] - a[9] * a[6] * a[15] + a[9] * a[7] * a[14] +
             a[13] * a[6] * a[11] - a[13] * a[7] * a[10];
    inv[4] = -a[4] * a[10] * a[15] + a[4] * a[11] * a[14] + a[8] * a[6] * a[15] - a[8] * a[7] * a[14] -
             a[12] * a[6] * a[11] + a[12] * a[7] * a[10];
    inv[8] = a[4] * a[9] * a[15] - a[4] * a[11] * a[13] - a[8] * a[5] * a[15] + a[8] * a[7] * a[13] +
             a[12] * a[5] * a[11] - a[12] * a[7] * a[9];
    inv[12] = -a[4] * a[9] * a[14] + a[4] * a[10] * a[13] + a[8] * a[5] * a[14] - a[8] * a[6] * a[13] -
              a[12] * a[5] * a[10] + a[12] * a[6] * a[9];
    inv[1] = -a[1] * a[10] * a[15] + a[1] * a[11] * a[14] + a[9] * a[2] * a[15] - a[9] * a[3] * a[14] -
             a[13] * a[2] * a[11] + a[13] * a[3] * a[10];
    inv[5] = a[0] * a[10] * a[15] - a[0] * a[11] * a[14] - a[8] * a[2] * a[15] + a[8] * a[3] * a[14] +
             a[12] * a[2] * a[11] - a[12] * a[3] * a[10];
    inv[9] = -a[0] * a[9] * a[15] + a[0] * a[11] * a[13] + a[8] * a[1] * a[15] - a[8] * a[3] * a[13] -
             a[12] * a[1] * a[11] + a[12] * a[3] * a[9];
    inv[13] = a[0] * a[9] * a[14] - a[0] * a[10] * a[13] - a[8] * a[1] * a[14] + a[8] * a[2] * a[13] +
              a[12] * a[1] * a[10] - a[12] * a[2] * a[9];
    inv[2] = a[1] * a[6] * a[15] - a[1] * a[7] * a[14] - a[5] * a[2] * a[15] + a[5] * a[3] * a[14] +
             a[13] * a[2] * a[7] - a[13] * a[3] * a[6];
    inv[6] = -a[0] * a[6] * a[15] + a[0] * a[7] * a[14] + a[4] * a[2] * a[15] - a[4] * a[3] * a[14] -
             a[12] * a[2] * a[7] + a[12] * a[3] * a[6];
    inv[10] = a[0] * a[5] * a[15] - a[0] * a[7] * a[13] - a[4] * a[1] * a[15] + a[4] * a[3] * a[13] +
              a[12] * a[1] * a[7] - a[12] * a[3] * a[5];
    inv[14] = -a[0] * a[5] * a[14] + a[0] * a[6] * a[13] + a[4] * a[1] * a[14] - a[4] * a[2] * a[13] -
              a[12] * a[1] * a[6] + a[12] * a[2] * a[5];
    inv[3] = -a[1] * a[6] * a[11] + a[1] * a[7] * a[10] + a[5] * a[2] * a[11] - a[5] * a[3] * a[10] -
             a[9] * a[2] * a[7] + a[9] * a[3] * a[6];
    inv[7] = a[0] * a[6] * a[11] - a[0] * a[7] * a[10] - a[4] * a[2] * a[11] + a[4] * a[3] * a[10] +
             a[8] * a[2] * a[7] - a[8] * a[3] * a[6];
    inv[11] = -a[0] * a[5] * a[11] + a[0] * a[7] * a[9] + a[4] * a[1] * a[11] - a[4] * a[3] * a[9] -
              a[8] * a[1] * a[7] + a[8] * a[3] * a[5];
    inv[15] = a[0] * a[5] * a[10] - a[0] * a[6] * a[9] - a[4] * a[1] * a[10] + a[4] * a[2] * a[9] +
              a[8] * a[1] * a[6] - a[8] * a[2] * a[5];
    float det = a[0] * inv[0] + a[1] * inv[4] + a[2] * inv[8] + a[3] * inv[12];
    float invDet = det != 0.0F ? 1.0F / det : 0.0F;
    mat4 r;
    for (int col = 0; col < 4; ++col) {
        for (int row = 0; row < 4; ++row) {
            r[col][row] = inv[col * 4 + row] * invDet;
        }
    }
    return r;
}

// ---- quaternions (w, x, y, z constructor order) ------------------------------
struct quat {
    float x, y, z, w;
    quat() : x(0), y(0), z(0), w(1) {}
    quat(float w_, float x_, float y_, float z_) : x(x_), y(y_), z(z_), w(w_) {}
    bool operator==(const quat&) const = default;
};

inline quat conjugate(const quat& q) { return quat(q.w, -q.x, -q.y, -q.z); }

inline vec3 operator*(const quat& q, const vec3& v) {
    vec3 u(q.x, q.y, q.z);
    vec3 uv = cross(u, v);
    vec3 uuv = cross(u, uv);
    return v + ((uv * q.w) + uuv) * 2.0F;
}

inline mat4 mat4_cast(const quat& q) {
    mat4 r(1.0F);
    float xx = q.x * q.x, yy = q.y * q.y, zz = q.z * q.z;
    float xz = q.x * q.z, xy = q.x * q.y, yz = q.y * q.z;
    float wx = q.w * q.x, wy = q.w * q.y, wz = q.w * q.z;
    r[0][0] = 1.0F - 2.0F * (yy + zz);
    r[0][1] = 2.0F * (xy + wz);
    r[0][2] = 2.0F * (xz - wy);
    r[1][0] = 2.0F * (xy - wz);
    r[1][1] = 1.0F - 2.0F * (xx + zz);
    r[1][2] = 2.0F * (yz + wx);
    r[2][0] = 2.0F * (xz + wy);
    r[2][1] = 2.0F * (yz - wx);
    r[2][2] = 1.0F - 2.0F * (xx + yy);
    return r;
}

} // namespace glm
