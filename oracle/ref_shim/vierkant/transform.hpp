// Stand-in for the reference's include/vierkant/transform.hpp, reduced to what
// src/intersection.cpp uses: transform_t (translation / rotation / scale), is_scale_uniform,
// mat4_cast and transform * point. TEST INFRASTRUCTURE ONLY (oracle build).
#pragma once
#include "math.hpp"

namespace vierkant
{

struct transform_t
{
    glm::vec3 translation = glm::vec3(0.f);
    glm::quat rotation = glm::quat(1, 0, 0, 0);
    glm::vec3 scale = glm::vec3(1.f);
};

inline bool is_scale_uniform(const transform_t &t) { return t.scale.x == t.scale.y && t.scale.x == t.scale.z; }

inline glm::mat4 mat4_cast(const transform_t &t)
{
    glm::mat4 m = glm::mat4_cast(t.rotation);
    m[0] = m[0] * t.scale.x;
    m[1] = m[1] * t.scale.y;
    m[2] = m[2] * t.scale.z;
    m[3] = glm::vec4(t.translation, 1.f);
    return m;
}

inline glm::vec3 operator*(const transform_t &t, const glm::vec3 &v)
{
    return t.rotation * (v * t.scale) + t.translation;
}

}// namespace vierkant
