// vierkant_gb/intersection.hpp -- C++20 value API over the C ABI's host intersection functions.
//
// Drop-in for the ray-primitive part of vierkant's include/vierkant/intersection.hpp: the same type
// names (Ray, Plane, Triangle, Sphere, AABB, OBB, ray_intersection, ray_triangle_intersection,
// REJECT / INTERSECT / INSIDE) and the same free functions intersect(...) with both argument orders,
// in namespace vierkant::gb so that both headers can be included side by side. Every result is
// bit-identical to the reference's src/intersection.cpp (the library restates it operation for
// operation). The functions are pure, thread-safe and allocate nothing; a non-zero status from the
// library (only possible for invalid arguments) is turned into vierkant::gb::error here, at the
// wrapper level -- nothing throws across the C ABI.
//
// Vectors are vierkant::gb::vec3 (three floats). Any type with float members x, y, z -- glm::vec3
// in the reference's code base -- converts to it implicitly, and as<V>() converts back.
#pragma once

#include <cmath>
#include <cstdint>
#include <limits>
#include <stdexcept>
#include <string>

#include "../vkg.h"

namespace vierkant::gb
{

//! a failed library call: the vkg_status and the library's message
class error : public std::runtime_error
{
public:
    error(vkg_status status, const std::string &what) : std::runtime_error(what), m_status(status) {}

    [[nodiscard]] vkg_status status() const { return m_status; }

private:
    vkg_status m_status;
};

inline void check(vkg_status status, const char *what)
{
    if(status != VKG_OK) { throw error(status, std::string(what) + " failed (vkg_status " + std::to_string(status) + ")"); }
}

struct vec3
{
    float x = 0.f, y = 0.f, z = 0.f;

    constexpr vec3() = default;

    constexpr vec3(float x_, float y_, float z_) : x(x_), y(y_), z(z_) {}

    constexpr explicit vec3(float s) : x(s), y(s), z(s) {}

    //! from any vector type with x, y, z members (glm::vec3)
    template<class V>
        requires requires(const V &v) {
            v.x;
            v.y;
            v.z;
        } && (!std::is_same_v<V, vec3>)
    constexpr vec3(const V &v) : x(float(v.x)), y(float(v.y)), z(float(v.z))
    {}

    template<class V>
    [[nodiscard]] constexpr V as() const
    {
        return V(x, y, z);
    }

    constexpr float &operator[](int i) { return (&x)[i]; }

    constexpr const float &operator[](int i) const { return (&x)[i]; }

    [[nodiscard]] const float *data() const { return &x; }

    constexpr bool operator==(const vec3 &) const = default;
};

// intersection.hpp:18-23
enum intersection_type
{
    REJECT = VKG_REJECT,
    INTERSECT = VKG_INTERSECT,
    INSIDE = VKG_INSIDE
};

// intersection.hpp:28-37
struct ray_intersection
{
    intersection_type type = REJECT;
    float distance = 0.f;

    ray_intersection(intersection_type theType, float theDistance = 0.0f) : type(theType), distance(theDistance) {}

    explicit operator intersection_type() const { return type; }

    explicit operator bool() const { return type; }
};

// intersection.hpp:43-51
struct ray_triangle_intersection : public ray_intersection
{
    float u = 0.f, v = 0.f;

    ray_triangle_intersection(intersection_type theType, float theDistance = 0.0f, float theU = 0.0f, float theV = 0.0f)
        : ray_intersection(theType, theDistance), u(theU), v(theV)
    {}
};

// intersection.hpp:145-170: the constructor normalises the direction (v * (1 / sqrt(dot(v, v))), as
// glm::normalize); assign the members directly to keep a direction as given
struct Ray
{
    vec3 origin;
    vec3 direction;

    Ray() = default;

    Ray(const vec3 &origin_, const vec3 &direction_) : origin(origin_), direction(normalize(direction_)) {}

    static vec3 normalize(const vec3 &v)
    {
        float s = 1.0f / std::sqrt(v.x * v.x + v.y * v.y + v.z * v.z);
        return {v.x * s, v.y * s, v.z * s};
    }
};

// Plane(float a, float b, float c, float d), intersection.hpp:179 / intersection.cpp:196-201. The
// coefficients are kept as given; the library normalises them as the reference's constructor does.
struct Plane
{
    float coefficients[4] = {0.f, 1.f, 0.f, 0.f};

    Plane() = default;

    Plane(float a, float b, float c, float d) : coefficients{a, b, c, d} {}
};

// intersection.hpp:205-228
struct Triangle
{
    vec3 v0, v1, v2;

    const vec3 &operator[](int i) const { return (&v0)[i]; }

    vec3 &operator[](int i) { return (&v0)[i]; }
};

// intersection.hpp:230-245
struct Sphere
{
    vec3 center = {};
    float radius = 0.f;

    Sphere() = default;

    Sphere(const vec3 &c, float r) : center(c), radius(r) {}
};

struct AABB;
ray_intersection intersect(const AABB &aabb, const Ray &ray);

// intersection.hpp:281-350 (the parts a ray query needs)
struct AABB
{
    vec3 min = vec3(std::numeric_limits<float>::max());
    vec3 max = vec3(std::numeric_limits<float>::lowest());

    AABB() = default;

    AABB(const vec3 &theMin, const vec3 &theMax) : min(theMin), max(theMax) {}

    [[nodiscard]] bool valid() const { return max.x >= min.x && max.y >= min.y && max.z >= min.z; }

    inline explicit operator bool() const { return valid(); }

    //! AABB::intersect(const Ray&), intersection.hpp:349
    [[nodiscard]] ray_intersection intersect(const Ray &ray) const { return vierkant::gb::intersect(*this, ray); }
};

// intersection.hpp:352-357: centre, three axes (the columns of the reference's glm::mat3 axis) and
// half lengths along them
struct OBB
{
    vec3 center{};
    vec3 axis[3] = {vec3(1, 0, 0), vec3(0, 1, 0), vec3(0, 0, 1)};
    vec3 half_lengths{};
};

/********************************** Ray intersection tests ****************************************/

//! intersection.hpp:74 / intersection.cpp:10-21
inline ray_intersection intersect(const Plane &plane, const Ray &ray)
{
    vkg_ray_intersection r{};
    check(vkg_intersect_ray_plane(ray.origin.data(), ray.direction.data(), plane.coefficients, &r),
          "vkg_intersect_ray_plane");
    return {intersection_type(r.type), r.distance};
}

inline ray_intersection intersect(const Ray &ray, const Plane &plane) { return intersect(plane, ray); }

//! intersection.hpp:79 / intersection.cpp:114-129 (Moeller-Trumbore, two-sided, no t range)
inline ray_triangle_intersection intersect(const Triangle &triangle, const Ray &ray)
{
    float tri[9] = {triangle.v0.x, triangle.v0.y, triangle.v0.z, triangle.v1.x, triangle.v1.y,
                    triangle.v1.z, triangle.v2.x, triangle.v2.y, triangle.v2.z};
    vkg_ray_triangle_intersection r{};
    check(vkg_intersect_ray_triangle(ray.origin.data(), ray.direction.data(), tri, &r), "vkg_intersect_ray_triangle");
    return {intersection_type(r.type), r.distance, r.u, r.v};
}

inline ray_triangle_intersection intersect(const Ray &ray, const Triangle &triangle)
{
    return intersect(triangle, ray);
}

//! intersection.hpp:85 / intersection.cpp:133-148
inline ray_intersection intersect(const Sphere &sphere, const Ray &ray)
{
    vkg_ray_intersection r{};
    check(vkg_intersect_ray_sphere(ray.origin.data(), ray.direction.data(), sphere.center.data(), sphere.radius, &r),
          "vkg_intersect_ray_sphere");
    return {intersection_type(r.type), r.distance};
}

inline ray_intersection intersect(const Ray &ray, const Sphere &sphere) { return intersect(sphere, ray); }

//! intersection.hpp:90 / intersection.cpp:308-312 (slab test through the identity OBB)
inline ray_intersection intersect(const AABB &aabb, const Ray &ray)
{
    vkg_ray_intersection r{};
    check(vkg_intersect_ray_aabb(ray.origin.data(), ray.direction.data(), aabb.min.data(), aabb.max.data(), &r),
          "vkg_intersect_ray_aabb");
    return {intersection_type(r.type), r.distance};
}

inline ray_intersection intersect(const Ray &ray, const AABB &aabb) { return intersect(aabb, ray); }

//! intersection.hpp:95 / intersection.cpp:152-184
inline ray_intersection intersect(const OBB &obb, const Ray &ray)
{
    float axes[9];
    for(int a = 0; a < 3; ++a)
    {
        for(int k = 0; k < 3; ++k) { axes[3 * a + k] = obb.axis[a][k]; }
    }
    vkg_ray_intersection r{};
    check(vkg_intersect_ray_obb(ray.origin.data(), ray.direction.data(), obb.center.data(), axes,
                                obb.half_lengths.data(), &r),
          "vkg_intersect_ray_obb");
    return {intersection_type(r.type), r.distance};
}

inline ray_intersection intersect(const Ray &ray, const OBB &obb) { return intersect(obb, ray); }

/********************************** Triangle intersection tests ****************************************/

//! intersection.hpp:101 / intersection.cpp:364-370 (Akenine-Moeller separating axes)
inline uint32_t intersect(const Triangle &t, const AABB &b)
{
    float tri[9] = {t.v0.x, t.v0.y, t.v0.z, t.v1.x, t.v1.y, t.v1.z, t.v2.x, t.v2.y, t.v2.z};
    uint32_t out = 0;
    check(vkg_intersect_triangle_aabb(tri, b.min.data(), b.max.data(), &out), "vkg_intersect_triangle_aabb");
    return out;
}

inline uint32_t intersect(const AABB &b, const Triangle &t) { return intersect(t, b); }

//! intersection.hpp:105 / intersection.cpp:374-378 (Guigue-Devillers)
inline uint32_t intersect(const Triangle &t1, const Triangle &t2)
{
    float a[9] = {t1.v0.x, t1.v0.y, t1.v0.z, t1.v1.x, t1.v1.y, t1.v1.z, t1.v2.x, t1.v2.y, t1.v2.z};
    float b[9] = {t2.v0.x, t2.v0.y, t2.v0.z, t2.v1.x, t2.v1.y, t2.v1.z, t2.v2.x, t2.v2.y, t2.v2.z};
    uint32_t out = 0;
    check(vkg_intersect_triangle_triangle(a, b, &out), "vkg_intersect_triangle_triangle");
    return out;
}

}// namespace vierkant::gb
