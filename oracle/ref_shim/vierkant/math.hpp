// Stand-in for the reference's include/vierkant/math.hpp (which only pulls in glm headers):
// routes to the project-written linear-algebra shim. TEST INFRASTRUCTURE ONLY (oracle build).
#pragma once
#include "../glm_shim.hpp"
