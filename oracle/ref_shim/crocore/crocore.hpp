// Stand-in for crocore/crocore.hpp (empty submodule in the reference checkout): only
// crocore::mean, used by compute_centroid. TEST INFRASTRUCTURE ONLY (oracle build).
#pragma once
#include <vector>
#include "../glm_shim.hpp"

namespace crocore
{
inline glm::vec3 mean(const std::vector<glm::vec3> &values)
{
    glm::vec3 sum(0.f);
    for(const auto &v: values) { sum += v; }
    return values.empty() ? sum : sum / static_cast<float>(values.size());
}
}// namespace crocore
