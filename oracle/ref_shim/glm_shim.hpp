// Minimal linear-algebra shim that lets the reference's own src/intersection.cpp and
// src/triangle_intersection.h compile without the glm submodule (which is empty in the
// reference checkout). TEST INFRASTRUCTURE ONLY: this is part of the oracle build.
//
// Written from the GLSL / linear-algebra definitions (column-major matrices, m[c][r]),
// not from glm's sources. The arithmetic that matters for parity follows the published
// glm semantics (g-truc/glm; the pinned submodule commit is not recoverable):
//   dot(a, b)    = (a.x*b.x + a.y*b.y) + a.z*b.z      (left-to-right, no fusion)
//   cross(a, b)  = (a.y*b.z - b.y*a.z, a.z*b.x - b.z*a.x, a.x*b.y - b.x*a.y)
//   normalize(v) = v * (1 / sqrt(dot(v, v)))           (glm: v * inversesqrt(dot(v, v)))
// The oracle is compiled with -ffp-contract=off so no multiply-add is fused.
#pragma once

#include <cassert>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <limits>
#include <utility>

namespace glm
{

struct vec4;

struct vec2
{
    float x = 0.f, y = 0.f;
    constexpr vec2() = default;
    constexpr explicit vec2(float s) : x(s), y(s) {}
    constexpr vec2(float a, float b) : x(a), y(b) {}
    float &operator[](int i) { return (&x)[i]; }
    const float &operator[](int i) const { return (&x)[i]; }
};

struct vec3
{
    float x = 0.f, y = 0.f, z = 0.f;
    constexpr vec3() = default;
    constexpr explicit vec3(float s) : x(s), y(s), z(s) {}
    constexpr vec3(float a, float b, float c) : x(a), y(b), z(c) {}
    vec3(const vec4 &v);// implicit truncation, as in glm's non-explicit ctor mode
    float &operator[](int i) { return (&x)[i]; }
    const float &operator[](int i) const { return (&x)[i]; }
    vec3 &operator+=(const vec3 &o) { x = x + o.x; y = y + o.y; z = z + o.z; return *this; }
    vec3 &operator-=(const vec3 &o) { x = x - o.x; y = y - o.y; z = z - o.z; return *this; }
    vec3 &operator*=(const vec3 &o) { x = x * o.x; y = y * o.y; z = z * o.z; return *this; }
    vec3 &operator*=(float s) { x = x * s; y = y * s; z = z * s; return *this; }
    vec3 &operator/=(float s) { x = x / s; y = y / s; z = z / s; return *this; }
    bool operator==(const vec3 &o) const { return x == o.x && y == o.y && z == o.z; }
    bool operator!=(const vec3 &o) const { return !(*this == o); }
};

struct vec4
{
    float x = 0.f, y = 0.f, z = 0.f, w = 0.f;
    constexpr vec4() = default;
    constexpr explicit vec4(float s) : x(s), y(s), z(s), w(s) {}
    constexpr vec4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
    constexpr vec4(const vec3 &v, float d) : x(v.x), y(v.y), z(v.z), w(d) {}
    float &operator[](int i) { return (&x)[i]; }
    const float &operator[](int i) const { return (&x)[i]; }
    vec3 xyz() const { return {x, y, z}; }
    vec4 &operator/=(float s) { x = x / s; y = y / s; z = z / s; w = w / s; return *this; }
    vec4 &operator*=(float s) { x = x * s; y = y * s; z = z * s; w = w * s; return *this; }
    bool operator==(const vec4 &o) const { return x == o.x && y == o.y && z == o.z && w == o.w; }
};

inline vec3::vec3(const vec4 &v) : x(v.x), y(v.y), z(v.z) {}

// ---- vec3 arithmetic -------------------------------------------------------------------------
inline vec3 operator+(const vec3 &a, const vec3 &b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline vec3 operator-(const vec3 &a, const vec3 &b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline vec3 operator*(const vec3 &a, const vec3 &b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
inline vec3 operator/(const vec3 &a, const vec3 &b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
inline vec3 operator*(const vec3 &a, float s) { return {a.x * s, a.y * s, a.z * s}; }
inline vec3 operator*(float s, const vec3 &a) { return {s * a.x, s * a.y, s * a.z}; }
inline vec3 operator/(const vec3 &a, float s) { return {a.x / s, a.y / s, a.z / s}; }
inline vec3 operator+(const vec3 &a, float s) { return {a.x + s, a.y + s, a.z + s}; }
inline vec3 operator-(const vec3 &a) { return {-a.x, -a.y, -a.z}; }

inline vec4 operator+(const vec4 &a, const vec4 &b) { return {a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w}; }
inline vec4 operator-(const vec4 &a, const vec4 &b) { return {a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w}; }
inline vec4 operator*(const vec4 &a, float s) { return {a.x * s, a.y * s, a.z * s, a.w * s}; }
inline vec4 operator/(const vec4 &a, float s) { return {a.x / s, a.y / s, a.z / s, a.w / s}; }
inline vec4 operator-(const vec4 &a) { return {-a.x, -a.y, -a.z, -a.w}; }

inline float dot(const vec3 &a, const vec3 &b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float dot(const vec4 &a, const vec4 &b) { return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w; }
inline vec3 cross(const vec3 &a, const vec3 &b)
{
    return {a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y};
}
inline float length(const vec3 &v) { return std::sqrt(dot(v, v)); }
inline float length(const vec4 &v) { return std::sqrt(dot(v, v)); }
inline float length2(const vec3 &v) { return dot(v, v); }
inline float length2(const vec4 &v) { return dot(v, v); }
inline vec3 normalize(const vec3 &v) { return v * (1.f / std::sqrt(dot(v, v))); }
inline vec4 normalize(const vec4 &v) { return v * (1.f / std::sqrt(dot(v, v))); }
inline vec3 min(const vec3 &a, const vec3 &b)
{
    return {b.x < a.x ? b.x : a.x, b.y < a.y ? b.y : a.y, b.z < a.z ? b.z : a.z};
}
inline vec3 max(const vec3 &a, const vec3 &b)
{
    return {a.x < b.x ? b.x : a.x, a.y < b.y ? b.y : a.y, a.z < b.z ? b.z : a.z};
}
inline vec3 mix(const vec3 &a, const vec3 &b, float t) { return a * (1.f - t) + b * t; }

struct bvec3
{
    bool x, y, z;
};
inline bvec3 greaterThanEqual(const vec3 &a, const vec3 &b) { return {a.x >= b.x, a.y >= b.y, a.z >= b.z}; }
inline bool all(const bvec3 &b) { return b.x && b.y && b.z; }

inline float *value_ptr(vec3 &v) { return &v.x; }
inline const float *value_ptr(const vec3 &v) { return &v.x; }

template<typename T>
constexpr T half_pi()
{
    return T(1.57079632679489661923132169163975144);
}

// ---- matrices (column-major: m[c] is column c) --------------------------------------------
struct mat4;

struct mat3
{
    vec3 c[3];
    mat3() : c{vec3(0.f), vec3(0.f), vec3(0.f)} {}
    explicit mat3(float s) : c{vec3(s, 0, 0), vec3(0, s, 0), vec3(0, 0, s)} {}
    mat3(const vec3 &a, const vec3 &b, const vec3 &d) : c{a, b, d} {}
    explicit mat3(const mat4 &m);
    explicit mat3(const struct quat &q);
    vec3 &operator[](int i) { return c[i]; }
    const vec3 &operator[](int i) const { return c[i]; }
};

struct mat4
{
    vec4 c[4];
    mat4() : c{vec4(0.f), vec4(0.f), vec4(0.f), vec4(0.f)} {}
    explicit mat4(float s) : c{vec4(s, 0, 0, 0), vec4(0, s, 0, 0), vec4(0, 0, s, 0), vec4(0, 0, 0, s)} {}
    vec4 &operator[](int i) { return c[i]; }
    const vec4 &operator[](int i) const { return c[i]; }
};
using mat4x4 = mat4;

inline mat3::mat3(const mat4 &m) : c{m[0].xyz(), m[1].xyz(), m[2].xyz()} {}

inline vec3 operator*(const mat3 &m, const vec3 &v)
{
    return m[0] * v.x + m[1] * v.y + m[2] * v.z;
}
inline mat3 operator*(const mat3 &a, const mat3 &b) { return {a * b[0], a * b[1], a * b[2]}; }
inline vec4 operator*(const mat4 &m, const vec4 &v)
{
    return m[0] * v.x + m[1] * v.y + m[2] * v.z + m[3] * v.w;
}
inline mat4 operator*(const mat4 &a, const mat4 &b)
{
    mat4 r;
    for(int i = 0; i < 4; ++i) { r[i] = a * b[i]; }
    return r;
}

inline mat3 transpose(const mat3 &m)
{
    mat3 r;
    for(int i = 0; i < 3; ++i)
        for(int j = 0; j < 3; ++j) r[i][j] = m[j][i];
    return r;
}

inline mat3 inverse(const mat3 &m)
{
    // adjugate / determinant
    const float a = m[0][0], b = m[1][0], cc = m[2][0];
    const float d = m[0][1], e = m[1][1], f = m[2][1];
    const float g = m[0][2], h = m[1][2], i = m[2][2];
    const float A = e * i - f * h, B = -(d * i - f * g), C = d * h - e * g;
    const float det = a * A + b * B + cc * C;
    mat3 r;
    r[0][0] = A / det;
    r[0][1] = B / det;
    r[0][2] = C / det;
    r[1][0] = -(b * i - cc * h) / det;
    r[1][1] = (a * i - cc * g) / det;
    r[1][2] = -(a * h - b * g) / det;
    r[2][0] = (b * f - cc * e) / det;
    r[2][1] = -(a * f - cc * d) / det;
    r[2][2] = (a * e - b * d) / det;
    return r;
}

inline mat4 inverse(const mat4 &m)
{
    // Gauss-Jordan with partial pivoting on the row-major view of the matrix
    double a[4][8];
    for(int r = 0; r < 4; ++r)
        for(int c = 0; c < 4; ++c)
        {
            a[r][c] = m[c][r];
            a[r][c + 4] = (r == c) ? 1.0 : 0.0;
        }
    for(int col = 0; col < 4; ++col)
    {
        int piv = col;
        for(int r = col + 1; r < 4; ++r)
            if(std::fabs(a[r][col]) > std::fabs(a[piv][col])) piv = r;
        for(int k = 0; k < 8; ++k) std::swap(a[col][k], a[piv][k]);
        const double p = a[col][col];
        for(int k = 0; k < 8; ++k) a[col][k] /= p;
        for(int r = 0; r < 4; ++r)
        {
            if(r == col) continue;
            const double f = a[r][col];
            for(int k = 0; k < 8; ++k) a[r][k] -= f * a[col][k];
        }
    }
    mat4 out;
    for(int r = 0; r < 4; ++r)
        for(int c = 0; c < 4; ++c) out[c][r] = static_cast<float>(a[r][c + 4]);
    return out;
}

inline mat4 transpose(const mat4 &m)
{
    mat4 r;
    for(int i = 0; i < 4; ++i)
        for(int j = 0; j < 4; ++j) r[i][j] = m[j][i];
    return r;
}

inline mat3 inverseTranspose(const mat3 &m) { return transpose(inverse(m)); }
inline mat4 inverseTranspose(const mat4 &m) { return transpose(inverse(m)); }

// rotation of `m` by `angle` (radians) around `axis` (Rodrigues), applied on the right
inline mat4 rotate(const mat4 &m, float angle, const vec3 &axis)
{
    const float c = std::cos(angle), s = std::sin(angle);
    const vec3 u = normalize(axis);
    mat4 r(1.f);
    r[0] = vec4(c + u.x * u.x * (1 - c), u.y * u.x * (1 - c) + u.z * s, u.z * u.x * (1 - c) - u.y * s, 0);
    r[1] = vec4(u.x * u.y * (1 - c) - u.z * s, c + u.y * u.y * (1 - c), u.z * u.y * (1 - c) + u.x * s, 0);
    r[2] = vec4(u.x * u.z * (1 - c) + u.y * s, u.y * u.z * (1 - c) - u.x * s, c + u.z * u.z * (1 - c), 0);
    return m * r;
}

// ---- quaternion (w, x, y, z), unit quaternions only --------------------------------------
struct quat
{
    float w = 1.f, x = 0.f, y = 0.f, z = 0.f;
    constexpr quat() = default;
    constexpr quat(float w_, float x_, float y_, float z_) : w(w_), x(x_), y(y_), z(z_) {}
};

inline mat3 mat3_cast(const quat &q)
{
    const float xx = q.x * q.x, yy = q.y * q.y, zz = q.z * q.z;
    const float xy = q.x * q.y, xz = q.x * q.z, yz = q.y * q.z;
    const float wx = q.w * q.x, wy = q.w * q.y, wz = q.w * q.z;
    mat3 r;
    r[0] = vec3(1 - 2 * (yy + zz), 2 * (xy + wz), 2 * (xz - wy));
    r[1] = vec3(2 * (xy - wz), 1 - 2 * (xx + zz), 2 * (yz + wx));
    r[2] = vec3(2 * (xz + wy), 2 * (yz - wx), 1 - 2 * (xx + yy));
    return r;
}

inline vec3 operator*(const quat &q, const vec3 &v) { return mat3_cast(q) * v; }

inline mat3::mat3(const quat &q) : mat3(mat3_cast(q)) {}

inline mat4 mat4_cast(const quat &q)
{
    mat3 m = mat3_cast(q);
    mat4 r(1.f);
    for(int i = 0; i < 3; ++i) r[i] = vec4(m[i], 0.f);
    return r;
}

}// namespace glm
